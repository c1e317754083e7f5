// Forward projection y = A x (Joseph's method, one thread per ray).
//
// Replaces the FP half of ASTRA's cuda3d projector reached through
// ``astra.experimental.direct_FPBP3D(..., "FP")`` (tomosipo/astra.py:147-153).
//
// Data flow per call:
//  1. fp_layout_kernel writes, for every axis permutation (d, a, b) the angles
//     use, a zero-padded copy of the volume laid out [d][a][b] (b fastest).
//  2. fp_ray_kernel: one thread per (angle, row, column) walks the planes of
//     the dominant axis, samples bilinearly and scales by the plane step.
//     A warp is 32 consecutive detector rows of one column. b is the volume
//     axis det_v runs along, so the warp's samples on a plane lie on one short
//     run along b (contiguous in the copy); for circular and helical
//     geometries (det_v along z) all lanes also share the same two a columns.
//     Blocks are ordered row-fastest, then column, then angle. (Ordering by
//     row band across angles keeps a volume slab in L2 and wins at 384^3,
//     but measured slower at 512^3 / 1024 angles, the headline size.)
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace tsgb {
namespace {

constexpr int kFpRows = kFpTileRows;  // threads along detector rows (one warp)
constexpr int kFpCols = kFpTileCols;  // warps along detector columns

// Rays making more than ~89 degrees with the dominant axis are not sampled
// (both here and, through the weighted sinogram, in the transpose).
constexpr float kMaxSlope = 64.0f;

__global__ void fp_layout_kernel(const float* __restrict__ vol, float* __restrict__ out,
                                 LayoutDev L, long long s_d, long long s_a, long long s_b) {
  const long long n_ap = L.n_a + 2 * kPad;
  const long long n_bp = L.n_b + 2 * kPad;
  const long long total = (long long)L.n_d * n_ap * n_bp;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long jp = idx % n_bp;
    const long long rest = idx / n_bp;
    const long long ip = rest % n_ap;
    const long long k = rest / n_ap;
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
                                                 int k, int stride_d, int stride_a) {
  const float kt = float(k);
  const float qa = fmaf(kt, r.ma, r.Xa);
  const float qb = fmaf(kt, r.mb, r.Xb);
  const float fa0 = floorf(qa), fb0 = floorf(qb);
  const float fa = qa - fa0, fb = qb - fb0;
  const float* p = base + (k * stride_d + (int)fa0 * stride_a + (int)fb0);
  const float v00 = __ldg(p), v01 = __ldg(p + 1);
  const float v10 = __ldg(p + stride_a), v11 = __ldg(p + stride_a + 1);
  const float left = fmaf(fb, v01 - v00, v00);
  const float right = fmaf(fb, v11 - v10, v10);
  return fmaf(fa, right - left, left);
}

// Ray sum of pixel (iv, iu) at angle theta, already scaled by the plane step.
// W receives the plane step the transpose weights this ray with (0 for rays
// that are not sampled), exactly as bp_weight_kernel computes it.
__device__ __forceinline__ float fp_ray_total(const AngleParams& ap,
                                              const ColumnEntry* __restrict__ columns,
                                              const float* __restrict__ ws,
                                              const DeviceGeometry& g, int iv, int iu, int theta,
                                              float& W) {
  const float vt = float(iv - g.ov);
  const Ray r = ap.separable ? ray_column(columns[(size_t)theta * g.cols + iu], vt)
                             : ray_general(ap, float(iu - g.ou), vt);
  float total = 0.0f;
  W = 0.0f;
  if (finite_ray(r) && fabsf(r.ma) <= kMaxSlope && fabsf(r.mb) <= kMaxSlope) {
    W = ray_step(ap, r);
    const int o_d = ap.o_d, o_a = ap.o_a, o_b = ap.o_b;
    const int stride_d = ap.stride_d, stride_a = ap.stride_a;
    float klo = float(-o_d), khi = float(ap.n_d - 1 - o_d);
    clip_planes(r.Xa, r.ma, float(-1 - o_a), float(ap.n_a - o_a), klo, khi);
    clip_planes(r.Xb, r.mb, float(-1 - o_b), float(ap.n_b - o_b), klo, khi);
    if (klo <= khi) {
      const int k0 = (int)ceilf(klo), k1 = (int)floorf(khi);
      // base points at anchored voxel (0, 0, 0) of this copy
      const float* base = ws + ap.ws_offset + (long long)o_d * stride_d +
                          (long long)(o_a + kPad) * stride_a + (o_b + kPad);
      float acc0 = 0.0f, acc1 = 0.0f;
      int k = k0;
      for (; k < k1; k += 2) {
        acc0 += bilinear_sample(base, r, k, stride_d, stride_a);
        acc1 += bilinear_sample(base, r, k + 1, stride_d, stride_a);
      }
      if (k == k1) acc0 += bilinear_sample(base, r, k, stride_d, stride_a);
      total = (acc0 + acc1) * W;
    }
  }
  return total;
}

__global__ void __launch_bounds__(kFpRows* kFpCols)
    fp_ray_kernel(const AngleParams* __restrict__ params, const ColumnEntry* __restrict__ columns,
                  const float* __restrict__ ws, float* __restrict__ sino, DeviceGeometry g,
                  int angle0, int additive) {
  const int iv = blockIdx.x * kFpRows + threadIdx.x;
  const int iu = blockIdx.y * kFpCols + threadIdx.y;
  const int theta = angle0 + blockIdx.z;
  if (iu >= g.cols || iv >= g.rows) return;
  float W;
  const float total = fp_ray_total(params[theta], columns, ws, g, iv, iu, theta, W);
  float* out = sino + ((size_t)iv * g.nangles + theta) * g.cols + iu;
  if (additive)
    *out += total;
  else
    *out = total;
}

// ---------------------------------------------------------------- batched SIRT
// One launch over all jobs' (row block, column block, angle) tiles. Epilogue:
// residual = W * (R * (y - A x)), which is what the plain recipe computes with
// separate operations (y - A(x), times R, then the backprojector's W pass).
__global__ void __launch_bounds__(kFpRows* kFpCols)
    fp_sirt_batch_kernel(const SirtJobDev* __restrict__ jobs,
                         const long long* __restrict__ prefix, int n_jobs) {
  const long long b = blockIdx.x;
  const int j = find_job(prefix, n_jobs, b);
  const SirtJobDev& job = jobs[j];
  const DeviceGeometry& g = job.g;
  long long local = b - prefix[j];
  const int rb = int(local % job.fp_row_blocks);
  local /= job.fp_row_blocks;
  const int cb = int(local % job.fp_col_blocks);
  const int theta = int(local / job.fp_col_blocks);
  const int iv = rb * kFpRows + threadIdx.x;
  const int iu = cb * kFpCols + threadIdx.y;
  if (iu >= g.cols || iv >= g.rows) return;
  float W;
  const float total = fp_ray_total(job.params[theta], job.columns, job.fp_ws, g, iv, iu, theta, W);
  const size_t idx = ((size_t)iv * g.nangles + theta) * g.cols + iu;
  const float r = __fmul_rn(__fsub_rn(__ldg(job.y + idx), total), __ldg(job.R + idx));
  // res has kRowPad zero rows above and below the detector (never written)
  job.res[idx + (size_t)kRowPad * g.nangles * g.cols] = __fmul_rn(W, r);
}

// Layout copies of all jobs: blockIdx.y selects the (job, permutation) segment.
__global__ void fp_layout_batch_kernel(const LayoutSegDev* __restrict__ segs) {
  const LayoutSegDev& s = segs[blockIdx.y];
  const long long n_ap = s.n_a + 2 * kPad, n_bp = s.n_b + 2 * kPad;
  const long long total = (long long)s.n_d * n_ap * n_bp;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long jp = idx % n_bp, rest = idx / n_bp;
    const long long ip = rest % n_ap, k = rest / n_ap;
    const long long i = ip - kPad, jj = jp - kPad;
    float v = 0.0f;
    if (i >= 0 && i < s.n_a && jj >= 0 && jj < s.n_b)
      v = __ldg(s.vol + k * s.s_d + i * s.s_a + jj * s.s_b);
    s.out[idx] = v;
  }
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
    const long long total = L.n_d * (L.n_a + 2 * kPad) * (L.n_b + 2 * kPad);
    const int threads = 256;
    const long long blocks = (total + threads - 1) / threads;
    const int grid = int(blocks < 152LL * 64 ? blocks : 152LL * 64);
    fp_layout_kernel<<<grid, threads, 0, stream>>>(vol, workspace, lt.l[i], vstride[L.d],
                                                  vstride[L.a], vstride[L.b]);
  }
  const dim3 block(kFpRows, kFpCols);
  for (int a0 = 0; a0 < g.nangles; a0 += 65535) {
    const int n = g.nangles - a0 < 65535 ? g.nangles - a0 : 65535;
    const dim3 grid((g.rows + kFpRows - 1) / kFpRows, (g.cols + kFpCols - 1) / kFpCols, n);
    fp_ray_kernel<<<grid, block, 0, stream>>>(p->d_params, p->d_columns, workspace, sino, g, a0,
                                              additive ? 1 : 0);
  }
  return int(cudaGetLastError());
}

int launch_sirt_fp_batch(const SirtBatchDev& b, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  if (b.n_segs > 0) {
    const dim3 grid(unsigned(b.seg_grid_x), unsigned(b.n_segs));
    fp_layout_batch_kernel<<<grid, 256, 0, stream>>>(b.segs);
  }
  if (b.fp_blocks > 0)
    fp_sirt_batch_kernel<<<unsigned(b.fp_blocks), dim3(kFpRows, kFpCols), 0, stream>>>(
        b.jobs, b.fp_prefix, b.n_jobs);
  return int(cudaGetLastError());
}

}  // namespace tsgb
