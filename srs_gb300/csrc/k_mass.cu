// k_mass.cu — total Ca per compartment, accumulated in FP64.
//
// Total Ca of an element (uM): free Ca + Ca bound to every buffer state
// variable (ATP, calmodulin, troponin C, dye in the cytosol; calsequestrin in
// the JSR) + Ca bound to the rapid sarcolemmal buffers of UpdateFastBuffer
// (cpu/RunSimulation.cpp:15-22), which are at equilibrium with the free Ca:
// b_hi c / (K_hi + c) + b_lo c / (K_lo + c).  The rapid-buffer Euler form
// dc/dt = G / B with B = 1 + d(bound)/dc makes this the conserved quantity
// of the reaction and diffusion terms.  Per realization the kernel returns
// sum_j V0_j total_j (uM um^3) over the cytosol and over the JSR, summed in
// double precision whatever the precision of the state.
#include "srs_comp.h"
#include "srs_engine.h"

namespace srs {

__global__ void k_total_ca(MassArgs a) {
  const int r = blockIdx.x;
  double acc[2] = {0.0, 0.0};
  for (int e = threadIdx.x; e < a.n_state; e += blockDim.x) {
    const double v0 = a.v0[e];
    if (v0 == 0.0) continue;  // padding slot
    double c, bound;
    if (a.S64) {
      const double* S = a.S64 + (size_t)r * 6 * a.n_state;
      const size_t n = a.n_state;
      c = S[e];
      bound = S[n + e] + S[2 * n + e] + S[3 * n + e] + S[4 * n + e] + S[5 * n + e];
    } else {
      const size_t o = (size_t)r * a.n_state + e;
      const float4 m = a.M[o];
      const float im = a.I[o];
      float4 cm;
      float ci;
      if (a.CMq) {  // compact compensation (srs_comp.h)
        cm = comp_load4(a.CMq + o);
        ci = comp_load1(a.CIq[o]);
      } else {
        cm = a.CM[o];
        ci = a.CI[o];
      }
      const double* rs = a.rest4 + 4 * (size_t)e;
      c = rs[0] + ((double)m.x - (double)cm.x);
      bound = (rs[1] + ((double)m.y - (double)cm.y)) + (rs[2] + ((double)m.z - (double)cm.z)) +
              (rs[3] + ((double)m.w - (double)cm.w)) + (a.rest_imm[e] + ((double)im - (double)ci));
    }
    const double sl = a.bhi[e] * c / (a.khi + c) + a.blo[e] * c / (a.klo + c);
    acc[a.jsr[e] ? 1 : 0] += v0 * (c + bound + sl);
  }
  __shared__ double red[2][256];
  red[0][threadIdx.x] = acc[0];
  red[1][threadIdx.x] = acc[1];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[0][threadIdx.x] += red[0][threadIdx.x + s];
      red[1][threadIdx.x] += red[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.out[2 * r] = red[0][0];
    a.out[2 * r + 1] = red[1][0];
  }
}

int launch_total_ca(const MassArgs& a, int R, cudaStream_t st) {
  k_total_ca<<<R, 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// The compact compensation codec of srs_comp.h on the device: out[i] is in[i]
// after its round trip through the stored half.  Each thread takes five
// consecutive values, the first four through the four-species form (packed
// scalings when `packed`, as the plain adjoint stores them), the fifth
// through the single form.
__global__ void k_comp_round_trip(const float* in, float* out, int64_t n, int packed) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 5;
  if (i >= n) return;
  float v[5];
  for (int k = 0; k < 5; ++k) v[k] = i + k < n ? in[i + k] : 0.0f;
  ushort4 q;
  float4 c4;
  if (packed) {
    comp_store4_x2(&q, make_float4(v[0], v[1], v[2], v[3]));
    c4 = comp_load4_x2(&q);
  } else {
    comp_store4(&q, make_float4(v[0], v[1], v[2], v[3]));
    c4 = comp_load4(&q);
  }
  const float r[5] = {c4.x, c4.y, c4.z, c4.w, comp_load1(comp_store1(v[4]))};
  for (int k = 0; k < 5; ++k)
    if (i + k < n) out[i + k] = r[k];
}

int launch_comp_round_trip(const float* in, float* out, int64_t n, int packed, cudaStream_t st) {
  const int64_t groups = (n + 4) / 5;
  const int64_t blocks = (groups + 255) / 256;
  if (blocks > 0x7fffffff) return -1;
  k_comp_round_trip<<<(unsigned)blocks, 256, 0, st>>>(in, out, n, packed);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace srs
