// Detector supersampling (tomosipo/astra.py:80-98, doc/topics/operator.rst:69-86).
//
// With detector supersampling d the forward projection averages d x d rays
// per detector pixel, at sub-pixel offsets ((s + 0.5) / d - 0.5) pixels. Those
// are exactly the pixel centres of a d-times finer detector (rows * d x
// cols * d, pixel vectors det_v / d and det_u / d), so a supersampled
// projector runs its forward projection on that fine detector and bins each
// d x d block (times 1 / d^2); its matched backprojection spreads each pixel's
// value times 1 / d^2 over its block and backprojects on the fine detector,
// which is the exact transpose. Both passes are plain HBM copies.
#include <cuda_runtime.h>

#include "tsgb_internal.h"

namespace tsgb {
namespace {

// coarse[iv][t][iu] (+)= sum over the d x d block of fine, times 1 / d^2.
__global__ void ss_bin_kernel(const float* __restrict__ fine, float* __restrict__ coarse,
                              int rows, int nangles, int cols, int d, float scale, int additive) {
  const long long total = (long long)rows * nangles * cols;
  const long long fcols = (long long)cols * d;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long iu = idx % cols, rest = idx / cols;
    const long long t = rest % nangles, iv = rest / nangles;
    float s = 0.0f;
    for (int s1 = 0; s1 < d; ++s1) {
      const float* row = fine + ((iv * d + s1) * nangles + t) * fcols + iu * d;
      for (int s2 = 0; s2 < d; ++s2) s += __ldg(row + s2);
    }
    s *= scale;
    coarse[idx] = additive ? coarse[idx] + s : s;
  }
}

// fine[iv * d + s1][t][iu * d + s2] = coarse[iv][t][iu] / d^2.
__global__ void ss_expand_kernel(const float* __restrict__ coarse, float* __restrict__ fine,
                                 int rows, int nangles, int cols, int d, float scale) {
  const long long fcols = (long long)cols * d;
  const long long total = (long long)rows * d * nangles * fcols;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long fu = idx % fcols, rest = idx / fcols;
    const long long t = rest % nangles, fv = rest / nangles;
    fine[idx] = scale * __ldg(coarse + ((fv / d) * nangles + t) * cols + fu / d);
  }
}

int grid_for(long long total) {
  const long long blocks = (total + 255) / 256;
  return int(blocks < 152LL * 64 ? blocks : 152LL * 64);
}

}  // namespace

int launch_ss_bin(const tsgb_projector* p, const float* fine, float* coarse, bool additive,
                  void* stream) {
  const DeviceGeometry& g = p->g;
  const int d = p->det_ss;
  ss_bin_kernel<<<grid_for((long long)g.rows * g.nangles * g.cols), 256, 0,
                  static_cast<cudaStream_t>(stream)>>>(fine, coarse, g.rows, g.nangles, g.cols, d,
                                                       1.0f / float(d * d), additive ? 1 : 0);
  return int(cudaGetLastError());
}

int launch_ss_expand(const tsgb_projector* p, const float* coarse, float* fine, void* stream) {
  const DeviceGeometry& g = p->g;
  const int d = p->det_ss;
  ss_expand_kernel<<<grid_for((long long)g.rows * d * g.nangles * g.cols * d), 256, 0,
                     static_cast<cudaStream_t>(stream)>>>(coarse, fine, g.rows, g.nangles, g.cols,
                                                          d, 1.0f / float(d * d));
  return int(cudaGetLastError());
}

}  // namespace tsgb
