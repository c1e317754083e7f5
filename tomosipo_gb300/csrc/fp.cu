// Forward projection y = A x (Joseph's method, one thread per ray).
//
// Replaces the FP half of ASTRA's cuda3d projector reached through
// ``astra.experimental.direct_FPBP3D(..., "FP")`` (tomosipo/astra.py:147-153).
//
// Data flow per call:
//  1. fp_layout_transpose_kernel / fp_layout_kernel write, for every axis
//     permutation (d, a, b) the angles use, a zero-padded copy of the volume
//     laid out [d][a][b] (b fastest), as single voxels or as neighbour pairs
//     along b (the projector's tuning).
//  2. fp_ray_kernel: one thread per (row, column) and pair of adjacent angles
//     walks the planes of the dominant axis for both rays, samples
//     bilinearly and scales by the plane step. A warp is 32 consecutive
//     detector rows of one column. b is the volume axis det_v runs along, so
//     the warp's samples on a plane lie on one short run along b (contiguous
//     in the copy); for circular and helical geometries (det_v along z) all
//     lanes also share the same two a columns. Tiles run in the order of the
//     projector's schedule: groups of angle pairs over detector patches, so
//     the volume slab a group crosses stays in L2 (fp_schedule_tile).
#include <cuda_runtime.h>

#include <algorithm>

#include "device_common.cuh"

namespace tsgb {
namespace {

constexpr int kFpRows = kFpTileRows;  // threads along detector rows (one warp)
constexpr int kFpCols = kFpTileCols;  // warps along detector columns

// Rays making more than ~89 degrees with the dominant axis are not sampled
// (both here and, through the weighted sinogram, in the transpose).
constexpr float kMaxSlope = 64.0f;

// Padded copy c of the volume in an angle's [d][a][b] frame, c = 0 in the
// kPad-wide border (and past its far edge), stored as single voxels or as
// pairs along b: element (k, ip, jp) = (c[k][ip][jp], c[k][ip][jp+1]). Used
// when b is the volume's x, so reads and writes both run along x.
__device__ __forceinline__ float padded_voxel(const float* __restrict__ vol, const LayoutDev& L,
                                              long long k, long long ip, long long jp,
                                              long long s_d, long long s_a, long long s_b) {
  const long long i = ip - kPad, j = jp - kPad;
  if (i < 0 || i >= L.n_a || j < 0 || j >= L.n_b) return 0.0f;
  return __ldg(vol + k * s_d + i * s_a + j * s_b);
}

// Element of a padded copy: one voxel (float) or the pair (c[j], c[j+1]) along b
// (float2), as the projector's tuning chooses.
template <typename E>
__device__ __forceinline__ E copy_elem(float a, float b);
template <>
__device__ __forceinline__ float copy_elem<float>(float a, float) {
  return a;
}
template <>
__device__ __forceinline__ float2 copy_elem<float2>(float a, float b) {
  return make_float2(a, b);
}

template <typename E>
__global__ void fp_layout_kernel(const float* __restrict__ vol, E* __restrict__ out,
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
    out[L.offset + idx] = copy_elem<E>(padded_voxel(vol, L, k, ip, jp, s_d, s_a, s_b),
                                       padded_voxel(vol, L, k, ip, jp + 1, s_d, s_a, s_b));
  }
}

// The same copy when the volume's contiguous axis x is d or a (so b, the
// copy's fastest axis, is strided in the volume): each block transposes a
// 32 x 33 tile of the (f, b) plane through shared memory, where f is the copy
// axis that is x in the volume (f_is_d: f = d, else f = a), for one index t
// of the remaining copy axis per blockIdx.z step, and writes 32 elements
// along b (the 33rd b value is the last pair's second half). Reads run along x and
// writes along b, both coalesced. Coordinates are those of the padded copy.
template <typename E>
__global__ void __launch_bounds__(256)
    fp_layout_transpose_kernel(const float* __restrict__ vol, E* __restrict__ out,
                               LayoutDev L, long long s_d, long long s_a, long long s_b,
                               int f_is_d) {
  __shared__ float tile[33][33];  // [b][f]
  const int n_ap = L.n_a + 2 * kPad, n_bp = L.n_b + 2 * kPad;
  const int f_ext = f_is_d ? L.n_d : n_ap;
  const int t_ext = f_is_d ? n_ap : L.n_d;
  const int f0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  for (int t = blockIdx.z; t < t_ext; t += gridDim.z) {
    for (int r = threadIdx.y; r < 33; r += 8) {
      const int f = f0 + threadIdx.x, bp = b0 + r;
      const int k = f_is_d ? f : t, ip = f_is_d ? t : f;
      const int i = ip - kPad, j = bp - kPad;
      float v = 0.0f;
      if (f < f_ext && i >= 0 && i < L.n_a && j >= 0 && j < L.n_b)
        v = __ldg(vol + k * s_d + i * s_a + j * s_b);
      tile[r][threadIdx.x] = v;
    }
    __syncthreads();
#pragma unroll
    for (int r = threadIdx.y; r < 32; r += 8) {
      const int f = f0 + r, bp = b0 + threadIdx.x;
      const int k = f_is_d ? f : t, ip = f_is_d ? t : f;
      if (f < f_ext && bp < n_bp)
        out[L.offset + ((long long)k * n_ap + ip) * n_bp + bp] =
            copy_elem<E>(tile[threadIdx.x][r], tile[threadIdx.x + 1][r]);
    }
    __syncthreads();
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

// floor(q) as an int and q - floor(q), without the conversion unit
// (kFloorMagic); identical to floorf. The sampled positions stay within a few
// voxels of the volume, far inside its |q| < 2^22 range.
struct FloorSplit {
  float frac;
  int i;
};
__device__ __forceinline__ FloorSplit floor_split(float q) {
  const float m = __fadd_rd(q, kFloorMagic);
  return {q - (m - kFloorMagic), int(__float_as_uint(m) - kFloorBits)};
}

// Bilinear sample of plane k from single voxels (four 4-byte taps) ...
__device__ __forceinline__ float bilinear_sample(const float* __restrict__ base, const Ray& r,
                                                 int k, int stride_d, int stride_a) {
  const float kt = float(k);
  const float qa = fmaf(kt, r.ma, r.Xa);
  const float qb = fmaf(kt, r.mb, r.Xb);
  const FloorSplit sa = floor_split(qa), sb = floor_split(qb);
  const float fa = sa.frac, fb = sb.frac;
  const float* p = base + (k * stride_d + sa.i * stride_a + sb.i);
  const float v00 = __ldg(p), v01 = __ldg(p + 1);
  const float v10 = __ldg(p + stride_a), v11 = __ldg(p + stride_a + 1);
  const float left = fmaf(fb, v01 - v00, v00);
  const float right = fmaf(fb, v11 - v10, v10);
  return fmaf(fa, right - left, left);
}

// ... or from pairs (two 8-byte taps, each holding both b neighbours); the
// arithmetic is the same, so both give identical results.
__device__ __forceinline__ float bilinear_sample(const float2* __restrict__ base, const Ray& r,
                                                 int k, int stride_d, int stride_a) {
  const float kt = float(k);
  const float qa = fmaf(kt, r.ma, r.Xa);
  const float qb = fmaf(kt, r.mb, r.Xb);
  const FloorSplit sa = floor_split(qa), sb = floor_split(qb);
  const float fa = sa.frac, fb = sb.frac;
  const float2* p = base + (k * stride_d + sa.i * stride_a + sb.i);
  const float2 v0 = __ldg(p), v1 = __ldg(p + stride_a);
  const float left = fmaf(fb, v0.y - v0.x, v0.x);
  const float right = fmaf(fb, v1.y - v1.x, v1.x);
  return fmaf(fa, right - left, left);
}

// The padded volume copy an angle samples: anchored voxel (0, 0, 0) and strides.
template <typename E>
struct CopyView {
  const E* base;
  int stride_d, stride_a;
};

template <typename E>
__device__ __forceinline__ CopyView<E> copy_view(const AngleParams& ap, const E* __restrict__ ws) {
  CopyView<E> v;
  v.stride_d = ap.stride_d;
  v.stride_a = ap.stride_a;
  v.base = ws + ap.ws_offset + (long long)ap.o_d * ap.stride_d +
           (long long)(ap.o_a + kPad) * ap.stride_a + (ap.o_b + kPad);
  return v;
}

// A ray's coefficients and the planes it samples (k0 > k1: none).
struct RaySpan {
  Ray r;
  int k0, k1;
};

__device__ __forceinline__ bool ray_sampled(const Ray& r) {
  return finite_ray(r) && fabsf(r.ma) <= kMaxSlope && fabsf(r.mb) <= kMaxSlope;
}

// Plane step the transpose weights a ray with (0 for rays that are not
// sampled), exactly as bp_weight_kernel computes it.
__device__ __forceinline__ float ray_weight(const AngleParams& ap, const Ray& r) {
  return ray_sampled(r) ? ray_step(ap, r) : 0.0f;
}

__device__ __forceinline__ RaySpan prepare_span(const AngleParams& ap,
                                                const ColumnEntry* __restrict__ columns,
                                                const DeviceGeometry& g, int iv, int iu,
                                                int theta) {
  RaySpan s;
  const float vt = float(iv - g.ov);
  s.r = ap.separable ? ray_column(columns[(size_t)theta * g.cols + iu], vt)
                     : ray_general(ap, float(iu - g.ou), vt);
  s.k0 = 1;
  s.k1 = 0;
  if (ray_sampled(s.r)) {
    float klo = float(-ap.o_d), khi = float(ap.n_d - 1 - ap.o_d);
    clip_planes(s.r.Xa, s.r.ma, float(-1 - ap.o_a), float(ap.n_a - ap.o_a), klo, khi);
    clip_planes(s.r.Xb, s.r.mb, float(-1 - ap.o_b), float(ap.n_b - ap.o_b), klo, khi);
    if (klo <= khi) {
      s.k0 = (int)ceilf(klo);
      s.k1 = (int)floorf(khi);
    }
  }
  return s;
}

template <typename E>
__device__ __forceinline__ float sample(const CopyView<E>& v, const Ray& r, int k) {
  return bilinear_sample(v.base, r, k, v.stride_d, v.stride_a);
}

// Samples of planes k0..k1 are summed into two partial sums by the parity of
// k (even planes into e, odd into o), in increasing k, so a ray's result does
// not depend on how its planes are scheduled against another ray's.
template <typename E>
__device__ __forceinline__ void walk(const CopyView<E>& v, const Ray& r, int k0, int k1, float& e,
                                     float& o) {
  int k = k0;
  if (k <= k1 && (k & 1)) o += sample(v, r, k++);
  for (; k < k1; k += 2) {
    e += sample(v, r, k);
    o += sample(v, r, k + 1);
  }
  if (k == k1) e += sample(v, r, k);
}

// Ray sum (scaled by the plane step) of pixel (iv, iu) at angle theta. If W
// is given it receives ray_weight. Values needed only after the plane loop
// are computed after it, which keeps registers free for loads in flight.
template <typename E>
__device__ __forceinline__ float fp_ray_total(const AngleParams& ap,
                                              const ColumnEntry* __restrict__ columns,
                                              const E* __restrict__ ws,
                                              const DeviceGeometry& g, int iv, int iu, int theta,
                                              float* W) {
  const RaySpan s = prepare_span(ap, columns, g, iv, iu, theta);
  float e = 0.0f, o = 0.0f;
  walk(copy_view(ap, ws), s.r, s.k0, s.k1, e, o);
  if (W) *W = ray_weight(ap, s.r);
  return s.k0 <= s.k1 ? (e + o) * ray_step(ap, s.r) : 0.0f;
}

// Two adjacent angles of one pixel. When both use the same volume copy their
// planes are walked together through one base pointer and one set of strides,
// so the second ray's taps (near the first's) hit lines the first just
// brought into L1. Results equal fp_ray_total's.
template <typename E>
__device__ __forceinline__ void fp_ray_pair(const AngleParams& apa, const AngleParams& apb,
                                            const ColumnEntry* __restrict__ columns,
                                            const E* __restrict__ ws,
                                            const DeviceGeometry& g, int iv, int iu, int theta,
                                            float& ta, float& tb, float* Wa, float* Wb) {
  const RaySpan a = prepare_span(apa, columns, g, iv, iu, theta);
  const RaySpan b = prepare_span(apb, columns, g, iv, iu, theta + 1);
  const CopyView<E> va = copy_view(apa, ws);
  float ea = 0.0f, oa = 0.0f, eb = 0.0f, ob = 0.0f;
  const int lo = max(a.k0, b.k0), hi = min(a.k1, b.k1);
  if (apa.layout == apb.layout && lo <= hi) {
    walk(va, a.r, a.k0, lo - 1, ea, oa);
    walk(va, b.r, b.k0, lo - 1, eb, ob);
    int k = lo;
    if (k & 1) {
      oa += sample(va, a.r, k);
      ob += sample(va, b.r, k);
      ++k;
    }
    for (; k < hi; k += 2) {
      ea += sample(va, a.r, k);
      eb += sample(va, b.r, k);
      oa += sample(va, a.r, k + 1);
      ob += sample(va, b.r, k + 1);
    }
    if (k == hi) {
      ea += sample(va, a.r, k);
      eb += sample(va, b.r, k);
    }
    walk(va, a.r, hi + 1, a.k1, ea, oa);
    walk(va, b.r, hi + 1, b.k1, eb, ob);
  } else {
    walk(va, a.r, a.k0, a.k1, ea, oa);
    walk(copy_view(apb, ws), b.r, b.k0, b.k1, eb, ob);
  }
  ta = a.k0 <= a.k1 ? (ea + oa) * ray_step(apa, a.r) : 0.0f;
  tb = b.k0 <= b.k1 ? (eb + ob) * ray_step(apb, b.r) : 0.0f;
  if (Wa) *Wa = ray_weight(apa, a.r);
  if (Wb) *Wb = ray_weight(apb, b.r);
}

// SIRT epilogue: residual W * (R * (y - A x)) of pixel idx, written where the
// backprojector reads it. s.res is the row-pair sinogram of bp_weight_kernel
// (kRowPad padding rows above and below the detector, zeroed once by the
// caller and never written): the pixel is the first value of its own row's
// pair and the second of the pair one row up. The plain recipe computes the
// same products with separate operations (y - A(x), times R, then the
// backprojector's W pass), rounded the same way.
// With s.zlayout the pairs are column-major (bp_weight_z_kernel): pixel
// (iv, theta, iu) is the first value of pair (theta, iu, iv + kRowPad) and the
// second of the pair before it.
__device__ __forceinline__ void sirt_residual(const FpSirt& s, const DeviceGeometry& g,
                                              long long idx, float total, float W) {
  const float r = __fmul_rn(__fsub_rn(__ldg(s.y + idx), total), __ldg(s.R + idx));
  const float v = __fmul_rn(W, r);
  if (s.zlayout) {
    const long long iu = idx % g.cols, rest = idx / g.cols;
    const long long theta = rest % g.nangles, iv = rest / g.nangles;
    float* e = s.res + 2 * ((theta * g.cols + iu) * (g.rows + 2 * kRowPad) + iv + kRowPad);
    e[0] = v;
    e[-1] = v;
    return;
  }
  const long long rs = (long long)g.nangles * g.cols;
  float* e = s.res + 2 * (idx + kRowPad * rs);
  e[0] = v;
  e[1 - 2 * rs] = v;
}

// One thread per pixel and pair of adjacent angles; the linear block index
// is mapped to a tile by the projector's schedule. The output offset and the
// pair flag wait in shared memory during the walk (volatile, so they are not
// kept in registers across it). Four resident blocks per SM leave 64
// registers a thread, which the plane loop spends on loads in flight.
// kSirt: write the SIRT residual (sirt_residual) instead of the sinogram.
// E: the copies' element type (float: single voxels, float2: pairs along b).
// One tile (the schedule's block `block`) of the forward projection; the body
// of fp_ray_kernel and of fp_ray_multi_kernel. out_slot: the block's shared
// parking slots (one per thread).
template <bool kSirt, typename E>
__device__ __forceinline__ void fp_ray_tile(const AngleParams* __restrict__ params,
                                            const ColumnEntry* __restrict__ columns,
                                            const E* __restrict__ ws, float* __restrict__ sino,
                                            const DeviceGeometry& g, const FpSchedule& sched,
                                            int angle0, int angle_end, int additive,
                                            const FpSirt& sirt, long long block,
                                            volatile long long* out_slot) {
  int rb, cb, pr;
  fp_schedule_tile(sched, block, rb, cb, pr);
  const int iv = rb * kFpRows + threadIdx.x;
  const int iu = cb * kFpCols + threadIdx.y;
  const int theta = angle0 + 2 * pr;
  if (iu >= g.cols || iv >= g.rows) return;
  const int slot = threadIdx.y * kFpRows + threadIdx.x;
  // the launch covers angles angle0 .. angle_end - 1: an odd count leaves the
  // last thread one angle
  const bool pair_in = theta + 1 < angle_end;
  out_slot[slot] = (((long long)iv * g.nangles + theta) * g.cols + iu) * 2 + (pair_in ? 1 : 0);
  float ta, tb = 0.0f, Wa = 0.0f, Wb = 0.0f;
  if (pair_in)
    fp_ray_pair(params[theta], params[theta + 1], columns, ws, g, iv, iu, theta, ta, tb,
                kSirt ? &Wa : nullptr, kSirt ? &Wb : nullptr);
  else
    ta = fp_ray_total(params[theta], columns, ws, g, iv, iu, theta, kSirt ? &Wa : nullptr);
  const long long packed = out_slot[slot];
  const bool pair = (packed & 1) != 0;
  const long long idx = packed >> 1;
  if (kSirt) {
    sirt_residual(sirt, g, idx, ta, Wa);
    if (pair) sirt_residual(sirt, g, idx + g.cols, tb, Wb);
  } else {
    float* out = sino + idx;
    if (additive) {
      out[0] += ta;
      if (pair) out[g.cols] += tb;
    } else {
      out[0] = ta;
      if (pair) out[g.cols] = tb;
    }
  }
}

template <bool kSirt, typename E>
__global__ void __launch_bounds__(kFpRows* kFpCols, 4)
    fp_ray_kernel(const AngleParams* __restrict__ params, const ColumnEntry* __restrict__ columns,
                  const E* __restrict__ ws, float* __restrict__ sino, DeviceGeometry g,
                  FpSchedule sched, int angle0, int angle_end, int additive, FpSirt sirt) {
  __shared__ volatile long long out_slot[kFpRows * kFpCols];
  fp_ray_tile<kSirt, E>(params, columns, ws, sino, g, sched, angle0, angle_end, additive, sirt,
                        blockIdx.x, out_slot);
}

// SIRT forward projections of many jobs in one launch: block b runs tile
// b - start[j] of job j, exactly as fp_ray_kernel would for that job alone.
template <bool kSirt, typename E>
__global__ void __launch_bounds__(kFpRows* kFpCols, 4)
    fp_ray_multi_kernel(const __grid_constant__ FpMulti m) {
  __shared__ volatile long long out_slot[kFpRows * kFpCols];
  const int j = multi_job_of(m.start, m.n, blockIdx.x);
  const FpMultiJob& J = m.job[j];
  fp_ray_tile<kSirt, E>(J.params, J.columns, static_cast<const E*>(J.ws), J.sino, J.g, J.sched,
                        0, J.g.nangles, J.additive, J.sirt, blockIdx.x - m.start[j], out_slot);
}

}  // namespace

namespace {

// Volume copies and ray kernels with copy elements of type E (offsets and
// strides count elements, so both types use the same plan).
template <typename E>
void launch_fp_elems(const tsgb_projector* p, const float* vol, float* sino, bool additive,
                     E* copies, cudaStream_t stream, const FpSirt* sirt, int angle_begin,
                     int angle_end, bool copies_ready) {
  const DeviceGeometry& g = p->g;
  const LayoutTable lt = make_layout_table(p);
  const long long vstride[3] = {(long long)g.ny * g.nx, (long long)g.nx, 1};
  for (int i = 0; i < lt.count && !copies_ready; ++i) {
    const Layout& L = p->layouts[i];
    if (L.b == 2) {  // b is x: a plain copy reads and writes along x
      const long long total = L.n_d * (L.n_a + 2 * kPad) * (L.n_b + 2 * kPad);
      const int threads = 256;
      const long long blocks = (total + threads - 1) / threads;
      const int grid = int(blocks < 152LL * 64 ? blocks : 152LL * 64);
      fp_layout_kernel<E><<<grid, threads, 0, stream>>>(vol, copies, lt.l[i], vstride[L.d],
                                                       vstride[L.a], vstride[L.b]);
    } else {
      const int f_is_d = L.d == 2 ? 1 : 0;  // which copy axis is the volume's x
      const long long f_ext = f_is_d ? L.n_d : L.n_a + 2 * kPad;
      const long long t_ext = f_is_d ? L.n_a + 2 * kPad : L.n_d;
      const dim3 grid(unsigned((f_ext + 31) / 32), unsigned((L.n_b + 2 * kPad + 31) / 32),
                      unsigned(t_ext < 65535 ? t_ext : 65535));
      fp_layout_transpose_kernel<E><<<grid, dim3(32, 8), 0, stream>>>(
          vol, copies, lt.l[i], vstride[L.d], vstride[L.a], vstride[L.b], f_is_d);
    }
  }
  const long long per_pair = (long long)((g.rows + kFpRows - 1) / kFpRows) *
                             ((g.cols + kFpCols - 1) / kFpCols);
  const long long chunk = fp_angle_chunk(g);
  for (long long a0 = angle_begin; a0 < angle_end; a0 += chunk) {
    const int n = int(angle_end - a0 < chunk ? angle_end - a0 : chunk);
    const FpSchedule s = fp_schedule(p, (n + 1) / 2);
    const long long blocks = per_pair * s.pairs;
    if (sirt)
      fp_ray_kernel<true, E><<<unsigned(blocks), dim3(kFpRows, kFpCols), 0, stream>>>(
          p->d_params, p->d_columns, copies, sino, g, s, int(a0), int(a0) + n, 0, *sirt);
    else
      fp_ray_kernel<false, E><<<unsigned(blocks), dim3(kFpRows, kFpCols), 0, stream>>>(
          p->d_params, p->d_columns, copies, sino, g, s, int(a0), int(a0) + n, additive ? 1 : 0,
          FpSirt{});
  }
}

}  // namespace

int launch_fp_copies(const tsgb_projector* p, const float* vol, float* workspace, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  // the copies only (no angles): launch_fp_elems with an empty angle range
  if (p->tuning.fp_pair_layout)
    launch_fp_elems(p, vol, nullptr, false, reinterpret_cast<float2*>(workspace), stream, nullptr,
                    0, 0, false);
  else
    launch_fp_elems(p, vol, nullptr, false, workspace, stream, nullptr, 0, 0, false);
  return int(cudaGetLastError());
}

bool fp_multi_eligible(const tsgb_projector* p) {
  const long long per_pair = (long long)((p->g.rows + kFpRows - 1) / kFpRows) *
                             ((p->g.cols + kFpCols - 1) / kFpCols);
  return p->g.nangles <= fp_angle_chunk(p->g) &&
         per_pair * ((p->g.nangles + 1) / 2) < (1LL << 31) / kMaxMultiJobs;
}

int launch_fp_multi(const FpMulti& m, bool pair_layout, void* stream_, bool sirt) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const long long blocks = m.start[m.n];
  if (blocks <= 0) return int(cudaGetLastError());
  const dim3 block(kFpRows, kFpCols);
  if (sirt && pair_layout)
    fp_ray_multi_kernel<true, float2><<<unsigned(blocks), block, 0, stream>>>(m);
  else if (sirt)
    fp_ray_multi_kernel<true, float><<<unsigned(blocks), block, 0, stream>>>(m);
  else if (pair_layout)
    fp_ray_multi_kernel<false, float2><<<unsigned(blocks), block, 0, stream>>>(m);
  else
    fp_ray_multi_kernel<false, float><<<unsigned(blocks), block, 0, stream>>>(m);
  return int(cudaGetLastError());
}

int launch_fp_batch(const tsgb_projector* p, const float* vol, float* sino, int64_t n,
                    bool additive, char* workspace, int64_t item_bytes, int group, void* stream) {
  const DeviceGeometry& g = p->g;
  const size_t vol_elems = size_t(g.nz) * g.ny * g.nx;
  const size_t sino_elems = size_t(g.rows) * g.nangles * g.cols;
  for (int64_t i0 = 0; i0 < n; i0 += group) {
    const int m = int(std::min<int64_t>(group, n - i0));
    FpMulti fm{};
    for (int k = 0; k < m; ++k) {
      float* ws = reinterpret_cast<float*>(workspace + k * item_bytes);
      const int rc = launch_fp_copies(p, vol + (i0 + k) * vol_elems, ws, stream);
      if (rc != 0) return rc;
      FpMultiJob& J = fm.job[k];
      J.params = p->d_params;
      J.columns = p->d_columns;
      J.ws = ws;
      J.g = g;
      J.sched = fp_schedule(p, (g.nangles + 1) / 2);
      J.sirt = FpSirt{};
      J.sino = sino + (i0 + k) * sino_elems;
      J.additive = additive ? 1 : 0;
      fm.start[k + 1] = fm.start[k] + fp_blocks(p);
    }
    fm.n = m;
    const int rc = launch_fp_multi(fm, p->tuning.fp_pair_layout != 0, stream, false);
    if (rc != 0) return rc;
  }
  return int(cudaGetLastError());
}

long long fp_blocks(const tsgb_projector* p) {
  const long long per_pair = (long long)((p->g.rows + kFpRows - 1) / kFpRows) *
                             ((p->g.cols + kFpCols - 1) / kFpCols);
  return per_pair * fp_schedule(p, (p->g.nangles + 1) / 2).pairs;
}

int launch_fp(const tsgb_projector* p, const float* vol, float* sino, bool additive,
              float* workspace, void* stream_, const FpSirt* sirt, int angle_begin,
              int angle_end, bool copies_ready) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  if (angle_end < 0) angle_end = p->g.nangles;
  if (p->tuning.fp_pair_layout)
    launch_fp_elems(p, vol, sino, additive, reinterpret_cast<float2*>(workspace), stream, sirt,
                    angle_begin, angle_end, copies_ready);
  else
    launch_fp_elems(p, vol, sino, additive, workspace, stream, sirt, angle_begin, angle_end,
                    copies_ready);
  return int(cudaGetLastError());
}

long long fp_angle_chunk(const DeviceGeometry& g) {
  // Angle chunks keep the forward projector's 1-D grid below 2^31 blocks.
  const long long per_pair = (long long)((g.rows + kFpRows - 1) / kFpRows) *
                             ((g.cols + kFpCols - 1) / kFpCols);
  const long long max_pairs = ((1LL << 31) - 1) / per_pair;
  return 2 * (max_pairs < (1LL << 29) ? max_pairs : (1LL << 29));
}

FpSchedule fp_schedule(const tsgb_projector* p, int pairs) {
  FpSchedule s;
  s.row_blocks = (p->g.rows + kFpRows - 1) / kFpRows;
  s.col_blocks = (p->g.cols + kFpCols - 1) / kFpCols;
  s.pairs = pairs;
  s.patch_rows = std::min(std::max(p->tuning.fp_patch_rows, 1), s.row_blocks);
  s.patch_cols = std::min(std::max(p->tuning.fp_patch_cols, 1), s.col_blocks);
  s.group_pairs = std::min(std::max(p->tuning.fp_group_pairs, 1), std::max(pairs, 1));
  return s;
}

tsgb_tuning default_tuning(const tsgb_projector* p) {
  tsgb_tuning t{};
  // Pairs along b halve the sampler's load instructions (the gather is bound
  // by L1 wavefronts) but double the copies' footprint: at 256^3 they are 11 %
  // faster, at 512^3 (a 1.1 GB pair copy) 12 % slower because the schedule's
  // volume slab then spills L2. Default: pairs while a pair copy is <= 512 MB.
  int64_t largest = 0;
  for (const auto& L : p->layouts) largest = std::max<int64_t>(largest, L.elems());
  t.fp_pair_layout = largest * 8 <= (int64_t(512) << 20) ? 1 : 0;
  // Patches of 256 detector rows x 32 columns and groups of 64 angles: the
  // volume slab such a group crosses stays in L2 while it runs (fastest on a
  // 512^3 cone scan with a 512 x 768 detector and 1024 angles, and within
  // 3 % of the fastest at 256^3 / 360 angles).
  t.fp_patch_rows = 256 / kFpRows;
  t.fp_patch_cols = 32 / kFpCols;
  t.fp_group_pairs = 32;
  // Matched backprojection: z-lane warps of 4 voxels x 16 z per lane x 8
  // planes for volumes of 448 or more voxels along z (512^3 / 1024 angles:
  // 124.8 ms against 144.5 ms for the voxel-pair kernel); below that a warp's
  // 512 z would leave lanes idle, and the voxel-pair kernel is faster at 256^3
  // (6.76 ms against 7.2 ms for the best z-lane shape).
  t.bp_kernel = p->g.nz >= 448 ? 1 : 0;
  t.bp_shape = 2;
  return t;
}


}  // namespace tsgb
