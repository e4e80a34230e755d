// k_linescan.cu — confocal line scan of the bound dye on the device.
//
// The reference's post-processing tool (linescan/main.cpp:197-225) forms, for
// each sample point x_i on a line, the PSF-weighted sum
//   F_i = sum_j V0_j * [CaDye]_j * N(r_ij; sigma)      (|r_ij|^2 < r_thresh)
// over mesh cells and padding voxels held at the resting fluorescence.  The
// host folds the cell volumes and PSF values into a sparse weight matrix
// (samples x elements, engine numbering) and the constant padding sum into an
// offset; this kernel evaluates the sum from the state in HBM for every
// realization, accumulating in double precision.
#include "srs_engine.h"

namespace srs {

// One block per (sample, realization).
__global__ void k_linescan(LinescanArgs a) {
  const int i = blockIdx.x, r = blockIdx.y;
  double acc = 0.0;
  for (int q = a.ptr[i] + threadIdx.x; q < a.ptr[i + 1]; q += blockDim.x) {
    const int e = a.col[q];
    double dye;
    if (a.S64) {
      dye = a.S64[(size_t)r * 6 * a.n_state + 5 * (size_t)a.n_state + e];
    } else {
      const size_t o = (size_t)r * a.n_state + e;
      const float u = a.M[o].w;
      const float c = a.CMq ? comp_load1(a.CMq[o].w) : a.CM[o].w;
      dye = a.rest_dye[e] + ((double)u - (double)c);
    }
    acc += a.w[q] * dye;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.out[(size_t)r * a.n_samples + i] = a.pad[i] + red[0];
}

int launch_linescan(const LinescanArgs& a, int R, cudaStream_t st) {
  dim3 grid(a.n_samples, R);
  k_linescan<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace srs
