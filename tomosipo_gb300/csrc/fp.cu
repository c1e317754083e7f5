// Forward projection y = A x (Joseph's method, one thread per ray).
//
// Replaces the FP half of ASTRA's cuda3d projector reached through
// ``astra.experimental.direct_FPBP3D(..., "FP")`` (tomosipo/astra.py:147-153).
//
// Data flow per call:
//  1. fp_layout_kernel writes, for every axis permutation (d, a, b) the angles
//     use, a zero-padded copy of the volume laid out [b][d][a] (a fastest).
//     Rays of one warp are adjacent detector columns, which move along a, so
//     their bilinear taps fall in the same cache lines.
//  2. fp_ray_kernel: one thread per (angle, row, column) walks the planes of
//     the dominant axis, samples bilinearly and scales by the plane step.
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace tsgb {
namespace {

constexpr int kFpCols = 32;  // threads along detector columns (one warp)
constexpr int kFpRows = 4;   // warps along detector rows

// Rays making more than ~89 degrees with the dominant axis are not sampled
// (both here and, through the weighted sinogram, in the transpose).
constexpr float kMaxSlope = 64.0f;

__global__ void fp_layout_kernel(const float* __restrict__ vol, float* __restrict__ out,
                                 LayoutDev L, long long s_d, long long s_a, long long s_b) {
  const long long n_ap = L.n_a + 2 * kPad;
  const long long n_bp = L.n_b + 2 * kPad;
  const long long total = n_bp * L.n_d * n_ap;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long ip = idx % n_ap;
    const long long rest = idx / n_ap;
    const long long k = rest % L.n_d;
    const long long jp = rest / L.n_d;
    const long long i = ip - kPad, j = jp - kPad;
    float v = 0.0f;
    if (i >= 0 && i < L.n_a && j >= 0 && j < L.n_b) v = __ldg(vol + k * s_d + i * s_a + j * s_b);
    out[L.offset + idx] = v;
  }
}

// Narrow [klo, khi] (plane coordinates) to planes where X + k m lies in (lo, hi).
__device__ __forceinline__ void clip_planes(float X, float m, float lo, float hi, float& klo,
                                            float& khi) {
  if (m != 0.0f) {
    const float inv = 1.0f / m;
    const float t1 = (lo - X) * inv, t2 = (hi - X) * inv;
    klo = fmaxf(klo, fminf(t1, t2));
    khi = fminf(khi, fmaxf(t1, t2));
  } else if (!(X > lo && X < hi)) {
    klo = 1.0f;
    khi = 0.0f;
  }
}

__device__ __forceinline__ float bilinear_sample(const float* __restrict__ base, const Ray& r,
                                                 int k, int stride_d, int stride_b) {
  const float kt = float(k);
  const float qa = fmaf(kt, r.ma, r.Xa);
  const float qb = fmaf(kt, r.mb, r.Xb);
  const float fa0 = floorf(qa), fb0 = floorf(qb);
  const float fa = qa - fa0, fb = qb - fb0;
  const float* p = base + ((int)fb0 * stride_b + k * stride_d + (int)fa0);
  const float v00 = __ldg(p), v01 = __ldg(p + 1);
  const float v10 = __ldg(p + stride_b), v11 = __ldg(p + stride_b + 1);
  const float top = fmaf(fa, v01 - v00, v00);
  const float bot = fmaf(fa, v11 - v10, v10);
  return fmaf(fb, bot - top, top);
}

__global__ void __launch_bounds__(kFpCols* kFpRows)
    fp_ray_kernel(const AngleParams* __restrict__ params, const ColumnEntry* __restrict__ columns,
                  const float* __restrict__ ws, float* __restrict__ sino, DeviceGeometry g,
                  int angle0, int additive) {
  const int iu = blockIdx.x * kFpCols + threadIdx.x;
  const int iv = blockIdx.y * kFpRows + threadIdx.y;
  const int theta = angle0 + blockIdx.z;
  if (iu >= g.cols || iv >= g.rows) return;
  const AngleParams& ap = params[theta];
  const float vt = float(iv - g.ov);
  const Ray r = ap.separable ? ray_column(columns[(size_t)theta * g.cols + iu], vt)
                             : ray_general(ap, float(iu - g.ou), vt);
  float total = 0.0f;
  if (finite_ray(r) && fabsf(r.ma) <= kMaxSlope && fabsf(r.mb) <= kMaxSlope) {
    const int o_d = ap.o_d, o_a = ap.o_a, o_b = ap.o_b;
    const int stride_d = ap.stride_d, stride_b = ap.stride_b;
    float klo = float(-o_d), khi = float(ap.n_d - 1 - o_d);
    clip_planes(r.Xa, r.ma, float(-1 - o_a), float(ap.n_a - o_a), klo, khi);
    clip_planes(r.Xb, r.mb, float(-1 - o_b), float(ap.n_b - o_b), klo, khi);
    if (klo <= khi) {
      const int k0 = (int)ceilf(klo), k1 = (int)floorf(khi);
      // base points at anchored voxel (0, 0, 0) of this copy
      const float* base = ws + ap.ws_offset + (long long)(o_b + kPad) * stride_b +
                          (long long)o_d * stride_d + (o_a + kPad);
      float acc0 = 0.0f, acc1 = 0.0f;
      int k = k0;
      for (; k < k1; k += 2) {
        acc0 += bilinear_sample(base, r, k, stride_d, stride_b);
        acc1 += bilinear_sample(base, r, k + 1, stride_d, stride_b);
      }
      if (k == k1) acc0 += bilinear_sample(base, r, k, stride_d, stride_b);
      total = (acc0 + acc1) * ray_step(ap, r);
    }
  }
  float* out = sino + ((size_t)iv * g.nangles + theta) * g.cols + iu;
  if (additive)
    *out += total;
  else
    *out = total;
}

}  // namespace

int launch_fp(const tsgb_projector* p, const float* vol, float* sino, bool additive,
              float* workspace, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const DeviceGeometry& g = p->g;
  const LayoutTable lt = make_layout_table(p);
  const long long vstride[3] = {(long long)g.ny * g.nx, (long long)g.nx, 1};
  for (int i = 0; i < lt.count; ++i) {
    const Layout& L = p->layouts[i];
    const long long total = (L.n_b + 2 * kPad) * L.n_d * (L.n_a + 2 * kPad);
    const int threads = 256;
    const long long blocks = (total + threads - 1) / threads;
    const int grid = int(blocks < 152LL * 64 ? blocks : 152LL * 64);
    fp_layout_kernel<<<grid, threads, 0, stream>>>(vol, workspace, lt.l[i], vstride[L.d],
                                                  vstride[L.a], vstride[L.b]);
  }
  const dim3 block(kFpCols, kFpRows);
  for (int a0 = 0; a0 < g.nangles; a0 += 65535) {
    const int n = g.nangles - a0 < 65535 ? g.nangles - a0 : 65535;
    const dim3 grid((g.cols + kFpCols - 1) / kFpCols, (g.rows + kFpRows - 1) / kFpRows, n);
    fp_ray_kernel<<<grid, block, 0, stream>>>(p->d_params, p->d_columns, workspace, sino, g, a0,
                                              additive ? 1 : 0);
  }
  return int(cudaGetLastError());
}

}  // namespace tsgb
