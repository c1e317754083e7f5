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

// A ray prepared for sampling: its coefficients, plane range and copy base.
struct RayWalk {
  Ray r;
  const float* base;  // anchored voxel (0, 0, 0) of the angle's padded copy
  int k0, k1;         // planes to sample (k0 > k1: none)
  int stride_d, stride_a;
  float W;            // plane step (0 if the ray is not sampled)
};

__device__ __forceinline__ RayWalk prepare_ray(const AngleParams& ap,
                                               const ColumnEntry* __restrict__ columns,
                                               const float* __restrict__ ws,
                                               const DeviceGeometry& g, int iv, int iu,
                                               int theta) {
  RayWalk w;
  const float vt = float(iv - g.ov);
  w.r = ap.separable ? ray_column(columns[(size_t)theta * g.cols + iu], vt)
                     : ray_general(ap, float(iu - g.ou), vt);
  w.k0 = 1;
  w.k1 = 0;
  w.W = 0.0f;
  w.stride_d = ap.stride_d;
  w.stride_a = ap.stride_a;
  w.base = ws + ap.ws_offset + (long long)ap.o_d * ap.stride_d +
           (long long)(ap.o_a + kPad) * ap.stride_a + (ap.o_b + kPad);
  if (finite_ray(w.r) && fabsf(w.r.ma) <= kMaxSlope && fabsf(w.r.mb) <= kMaxSlope) {
    w.W = ray_step(ap, w.r);
    float klo = float(-ap.o_d), khi = float(ap.n_d - 1 - ap.o_d);
    clip_planes(w.r.Xa, w.r.ma, float(-1 - ap.o_a), float(ap.n_a - ap.o_a), klo, khi);
    clip_planes(w.r.Xb, w.r.mb, float(-1 - ap.o_b), float(ap.n_b - ap.o_b), klo, khi);
    if (klo <= khi) {
      w.k0 = (int)ceilf(klo);
      w.k1 = (int)floorf(khi);
    }
  }
  return w;
}

__device__ __forceinline__ float sample(const RayWalk& w, int k) {
  return bilinear_sample(w.base, w.r, k, w.stride_d, w.stride_a);
}

// Samples of planes k0..k1 are summed into two partial sums by the parity of
// k (even planes into e, odd into o), in increasing k, so a ray's result does
// not depend on how its planes are scheduled against another ray's.
__device__ __forceinline__ void walk(const RayWalk& w, int k0, int k1, float& e, float& o) {
  int k = k0;
  if (k <= k1 && (k & 1)) o += sample(w, k++);
  for (; k < k1; k += 2) {
    e += sample(w, k);
    o += sample(w, k + 1);
  }
  if (k == k1) e += sample(w, k);
}

// Ray sum (scaled by the plane step) of pixel (iv, iu) at angle theta. W
// receives the plane step the transpose weights this ray with (0 for rays that
// are not sampled), exactly as bp_weight_kernel computes it.
__device__ __forceinline__ float fp_ray_total(const AngleParams& ap,
                                              const ColumnEntry* __restrict__ columns,
                                              const float* __restrict__ ws,
                                              const DeviceGeometry& g, int iv, int iu, int theta,
                                              float& W) {
  const RayWalk w = prepare_ray(ap, columns, ws, g, iv, iu, theta);
  W = w.W;
  float e = 0.0f, o = 0.0f;
  walk(w, w.k0, w.k1, e, o);
  return w.k0 <= w.k1 ? (e + o) * w.W : 0.0f;
}

// Two adjacent angles of one pixel. When both use the same volume copy their
// planes are walked together, so the second ray's taps (near the first's)
// hit lines the first just brought into L1. Results equal fp_ray_total's.
__device__ __forceinline__ void fp_ray_pair(const AngleParams& apa, const AngleParams& apb,
                                            const ColumnEntry* __restrict__ columns,
                                            const float* __restrict__ ws,
                                            const DeviceGeometry& g, int iv, int iu, int theta,
                                            float& ta, float& tb) {
  const RayWalk a = prepare_ray(apa, columns, ws, g, iv, iu, theta);
  const RayWalk b = prepare_ray(apb, columns, ws, g, iv, iu, theta + 1);
  float ea = 0.0f, oa = 0.0f, eb = 0.0f, ob = 0.0f;
  const int lo = max(a.k0, b.k0), hi = min(a.k1, b.k1);
  if (apa.layout == apb.layout && lo <= hi) {
    walk(a, a.k0, lo - 1, ea, oa);
    walk(b, b.k0, lo - 1, eb, ob);
    int k = lo;
    if (k & 1) {
      oa += sample(a, k);
      ob += sample(b, k);
      ++k;
    }
    for (; k < hi; k += 2) {
      ea += sample(a, k);
      eb += sample(b, k);
      oa += sample(a, k + 1);
      ob += sample(b, k + 1);
    }
    if (k == hi) {
      ea += sample(a, k);
      eb += sample(b, k);
    }
    walk(a, hi + 1, a.k1, ea, oa);
    walk(b, hi + 1, b.k1, eb, ob);
  } else {
    walk(a, a.k0, a.k1, ea, oa);
    walk(b, b.k0, b.k1, eb, ob);
  }
  ta = a.k0 <= a.k1 ? (ea + oa) * a.W : 0.0f;
  tb = b.k0 <= b.k1 ? (eb + ob) * b.W : 0.0f;
}

// One thread per pixel and pair of adjacent angles (blockIdx.z = pair).
__global__ void __launch_bounds__(kFpRows* kFpCols)
    fp_ray_kernel(const AngleParams* __restrict__ params, const ColumnEntry* __restrict__ columns,
                  const float* __restrict__ ws, float* __restrict__ sino, DeviceGeometry g,
                  int angle0, int additive) {
  const int iv = blockIdx.x * kFpRows + threadIdx.x;
  const int iu = blockIdx.y * kFpCols + threadIdx.y;
  const int theta = angle0 + 2 * blockIdx.z;
  if (iu >= g.cols || iv >= g.rows) return;
  float ta, tb = 0.0f, W;
  const bool pair = theta + 1 < g.nangles;
  if (pair)
    fp_ray_pair(params[theta], params[theta + 1], columns, ws, g, iv, iu, theta, ta, tb);
  else
    ta = fp_ray_total(params[theta], columns, ws, g, iv, iu, theta, W);
  float* out = sino + ((size_t)iv * g.nangles + theta) * g.cols + iu;
  if (additive) {
    out[0] += ta;
    if (pair) out[g.cols] += tb;
  } else {
    out[0] = ta;
    if (pair) out[g.cols] = tb;
  }
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
  for (int a0 = 0; a0 < g.nangles; a0 += 2 * 65535) {
    const int n = g.nangles - a0 < 2 * 65535 ? g.nangles - a0 : 2 * 65535;
    const dim3 grid((g.rows + kFpRows - 1) / kFpRows, (g.cols + kFpCols - 1) / kFpCols, (n + 1) / 2);
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
