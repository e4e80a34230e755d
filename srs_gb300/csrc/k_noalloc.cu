// k_noalloc.cu — an explicit step that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host application that owns every
// device allocation through its own pool or budget, or a real-time loop in
// which cudaMalloc/cudaFree (which may synchronise the device and take an
// unbounded time) must not run.  srs_explicit_step_fp64_noalloc serves them.
// The caller passes every input and output as its own device buffer; the only
// memory the step needs beyond those — the per-realization "blocks finished"
// counters and control blocks of the FP64 step kernel — lives in the
// fixed-size array below instead of in cudaMalloc'ed memory.
//
// The array exists once per GPU that loads this library and stays allocated
// until the process exits.  Every call shares it and it keeps the contents
// of the last call, so each call clears what must start at zero before its
// step.  Calls whose work overlaps on the GPU (different streams, or several
// host threads) race on the array: serialise them.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress) and caches it per device.
// That cache is not refreshed: cudaDeviceReset between calls is not
// supported (the cached address would belong to the destroyed context).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "srs_engine.h"
#include "srs_host.h"

namespace srs {

// Most realizations one call may advance (the array is sized for them).
constexpr int kNoallocMaxR = SRS_NOALLOC_MAX_REALIZATIONS;
struct NoallocLayout {
  unsigned int counters[kNoallocMaxR];
  RealCtl ctl[kNoallocMaxR];
};
constexpr size_t kNoallocBytes = (sizeof(NoallocLayout) + 255) & ~(size_t)255;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

struct NoallocInit {
  int32_t R;
  int64_t step;
  uint64_t seeds[kNoallocMaxR];
};

__global__ void k_noalloc_init(NoallocInit in, NoallocLayout* sc) {
  for (int r = threadIdx.x; r < in.R; r += blockDim.x) {
    sc->counters[r] = 0;
    RealCtl c;
    memset(&c, 0, sizeof(c));
    c.step = in.step;
    c.seed = in.seeds[r];
    c.lcc_close_step = -1;
    sc->ctl[r] = c;
  }
}

__global__ void k_noalloc_status(int32_t R, const NoallocLayout* sc, unsigned int* out) {
  unsigned int b = 0;
  for (int r = threadIdx.x; r < R; r += blockDim.x) b |= sc->ctl[r].status;
  if (b) atomicOr(out, b);
}

namespace {
std::mutex g_mtx;
void* g_addr[128] = {};  // symbol address of the array, per device

// Set-up on first use of a device: the device address of the array.  In host
// code `g_noalloc_scratch` names a host-side shadow, not device memory, so
// the address must come from cudaGetSymbolAddress with that device current.
int scratch_address(void** out, std::string* err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return SRS_ERR_CUDA;
  }
  if (dev < 0 || dev >= 128) {
    *err = "srs_explicit_step_fp64_noalloc supports devices 0..127, current device is " +
           std::to_string(dev);
    return SRS_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mtx);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return SRS_ERR_CUDA;
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return SRS_OK;
}
}  // namespace

}  // namespace srs

extern "C" const char* srs_last_error(void);
namespace srs {
int set_last_error(int code, const std::string& msg);
}

using namespace srs;

extern "C" int srs_explicit_step_fp64_noalloc(const srs_noalloc_step* d) {
  if (!d) return set_last_error(SRS_ERR_INPUT, "null argument");
  if (d->n_realizations <= 0 || d->n_realizations > kNoallocMaxR)
    return set_last_error(SRS_ERR_INPUT,
                          "srs_explicit_step_fp64_noalloc advances 1.." +
                              std::to_string(kNoallocMaxR) + " realizations per call, got " +
                              std::to_string(d->n_realizations));
  if (d->n_ele <= 0 || d->n_ryr < 0 || d->n_lcc < 0 || !d->reals || !d->seeds || !d->aij ||
      !d->nij || !d->br4 || !d->v0 || !d->bhi || !d->blo || !d->flags || !d->chan_ptr ||
      !d->states_in || !d->states_out || !d->ryr_states || !d->residuals ||
      !d->chan_list || (d->n_ryr > 0 && (!d->ryr_ele || !d->ryr_jsr)) ||
      (d->n_ryr > 0 && d->reals[R_RYR_A_STAR] != 0 && !d->ryr_nb) ||
      (d->n_lcc > 0 && (!d->lcc_states || !d->lccv_states || !d->lcc_ele)))
    return set_last_error(SRS_ERR_INPUT, "missing input or output pointer");
  if (d->n_ryr > 1024 && d->reals[R_RYR_A_STAR] != 0)
    return set_last_error(SRS_ERR_UNSUPPORTED, "coupled gating supports at most 1024 RyRs");
  void* base = nullptr;
  std::string err;
  int rc = scratch_address(&base, &err);
  if (rc) return set_last_error(rc, err);
  NoallocLayout* sc = reinterpret_cast<NoallocLayout*>(base);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(d->stream);

  srs_params ps;
  std::memset(&ps, 0, sizeof(ps));
  for (int i = 0; i < SRS_N_REAL_PARAMS; ++i) ps.reals[i] = d->reals[i];
  Plain64Args a;
  std::memset(&a, 0, sizeof(a));
  a.N = d->n_ele;
  a.R = d->n_realizations;
  a.aij = d->aij;
  a.nij = d->nij;
  a.br = d->br4;
  a.v0 = d->v0;
  a.bhi = d->bhi;
  a.blo = d->blo;
  a.flags = d->flags;
  a.chan_ptr = d->chan_ptr;
  a.chan_list = reinterpret_cast<const ChanEntry*>(d->chan_list);
  a.S_in = d->states_in;
  a.S_out = d->states_out;
  for (int q = 0; q < 56; ++q) a.p[q] = d->reals[q];
  a.nsr = d->ca_nsr;
  Protocol& P = a.P;
  gate_consts(ps, d->v_m, &P.gc[0]);
  P.gc[1] = P.gc[0];
  double Vg;
  lcc_flux_consts(ps, d->v_m, &P.lccA[0], &P.lccE[0], &P.lccEm1[0], &P.lccB, &Vg);
  P.lccA[1] = P.lccA[0];
  P.lccE[1] = P.lccE[0];
  P.lccEm1[1] = P.lccEm1[0];
  P.Vm[0] = P.Vm[1] = Vg;
  P.dt = d->reals[R_T_STEP];
  P.v_ryr = d->reals[R_V_RYR];
  P.v_cell = d->reals[R_V_CELL];
  P.nogating = d->nogating;
  P.run_protocol = 0;
  P.row_cap = 0;
  P.row_w = SRS_STATES_ROW_BASE;
  a.C.NR = d->n_ryr;
  a.C.NL = d->n_lcc;
  a.C.ryr_cleft = d->ryr_ele;
  a.C.ryr_jsr = d->ryr_jsr;
  a.C.ryr_nb = d->ryr_nb;
  a.C.lcc_ele = d->lcc_ele;
  a.CS.ryr = d->ryr_states;
  a.CS.lcc = d->lcc_states;
  a.CS.lccv = d->lccv_states;
  a.CS.res = d->residuals;
  a.CS.ctl = sc->ctl;
  a.CS.rows = nullptr;
  a.counters = sc->counters;

  NoallocInit in;
  std::memset(&in, 0, sizeof(in));
  in.R = d->n_realizations;
  in.step = d->step;
  for (int r = 0; r < d->n_realizations; ++r) in.seeds[r] = d->seeds[r];
  k_noalloc_init<<<1, 256, 0, st>>>(in, sc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_last_error(SRS_ERR_CUDA, std::string("init: ") + cudaGetErrorString(e));
  if (launch_plain64_step(a, st))
    return set_last_error(SRS_ERR_CUDA, std::string("step: ") + cudaGetErrorString(cudaGetLastError()));
  if (d->status) {
    k_noalloc_status<<<1, 256, 0, st>>>(d->n_realizations, sc, d->status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_last_error(SRS_ERR_CUDA, std::string("status: ") + cudaGetErrorString(e));
  }
  return SRS_OK;
}
