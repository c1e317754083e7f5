// Backprojection x = A^T y.
//
// Replaces the BP half of ASTRA's cuda3d projector reached through
// ``astra.experimental.direct_FPBP3D(..., "BP")`` (tomosipo/astra.py:147-153).
//
// Matched backprojection: the exact transpose of fp_ray_kernel, computed as a
// per-voxel gather (deterministic, no atomics). Voxel (k, i, j) in the
// angle's (d, a, b) frame receives W * y * tent(q_a - i) * tent(q_b - j) from
// every ray whose plane-k sample lies within one voxel of it.
//  1. bp_weight_kernel premultiplies the sinogram by each ray's plane step W
//     (the same W the forward projector applies) and stores it as row pairs,
//     (W y[v], W y[v+1]) per pixel, with zero padding rows.
//  2. bp_separable_kernel handles angles whose det_v lies along z (b = z):
//     q_a then depends on the column only, and on a plane of the dominant
//     axis a detector column's vertical profile does not depend on the
//     voxel's in-plane position. A thread owns two voxel columns adjacent
//     along the in-plane axis a and 16 voxels along z; per angle it solves
//     once for the columns that reach either and builds each column's
//     profile once per voxel, from one row-pair load. a is x for some angles
//     and y for others, so the angles run in two passes with different
//     thread-to-voxel mappings, the second adding onto the first.
//     (bp_zlane.cu holds the z-lane form of this step, with a column-major
//     weighted sinogram; the projector's tuning picks one.)
//  3. bp_general_kernel handles every other angle: it projects the corners of
//     the voxel's tent footprint onto the detector and tests every pixel in
//     their bounding box with the forward projector's own ray formula.
//
// Bilinear backprojection: voxel-driven, bilinear interpolation of the
// detector at the projected voxel centre, weighted so that it approximates
// the transpose (voxel volume / pixel area / ray obliquity, times the cone
// magnification squared). For z-flat geometries a quad copy of the sinogram
// gives each voxel its four taps in one load; the same kernel with FDK's
// weights is the backprojection of the FDK reconstruction.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "device_common.cuh"

namespace tsgb {
namespace {

constexpr float kMaxSlope = 64.0f;  // must match fp.cu
constexpr int kBpX = kBpTileX;      // threads along x (one warp)
constexpr int kBpY = kBpTileY;      // warps along y
constexpr int kRunZ = kBpRunZ;      // voxels along z per thread (matched)
constexpr int kRunZBil = 8;         // voxels along z per thread (bilinear)

// W * y of pixel (iv, iu) at angle theta (0 for rows outside the detector and
// for rays the forward projector does not sample). ce is the pixel's column
// entry (read only for separable angles).
__device__ __forceinline__ float weighted_pixel(const AngleParams& ap, const ColumnEntry& ce,
                                                const float* __restrict__ sino,
                                                const DeviceGeometry& g, int iv, int iu,
                                                int theta) {
  if (iv < 0 || iv >= g.rows) return 0.0f;
  const float vt = float(iv - g.ov);
  const Ray r = ap.separable ? ray_column(ce, vt) : ray_general(ap, float(iu - g.ou), vt);
  float w = 0.0f;
  if (finite_ray(r) && fabsf(r.ma) <= kMaxSlope && fabsf(r.mb) <= kMaxSlope) w = ray_step(ap, r);
  return w * __ldg(sino + ((size_t)iv * g.nangles + theta) * g.cols + iu);
}

// Row-pair weighted sinogram: element (iv, theta, iu) holds (W y[iv], W y[iv+1])
// for iv = -1 .. rows-1, so one 8-byte load gives the backprojector both rows
// of a tap. A thread walks kWeightRows consecutive pair rows of one detector
// column (threadIdx.y / blockIdx.y count them from iv = -1), loading the
// column's entry once and computing each row's W y once: the row's value is
// the second of one pair and the first of the next. Elements iv = -2, rows and
// rows+1 (the padding) are zeroed by the caller. `out` points at element
// (0, 0, 0); rows are nangles * cols elements apart.
constexpr int kWeightRows = 8;

__global__ void __launch_bounds__(256)
    bp_weight_kernel(const AngleParams* __restrict__ params,
                     const ColumnEntry* __restrict__ columns, const float* __restrict__ sino,
                     float2* __restrict__ out, DeviceGeometry g) {
  const int iu = blockIdx.x * 32 + threadIdx.x;
  const int r0 = (blockIdx.y * 8 + threadIdx.y) * kWeightRows - 1;
  const int theta = blockIdx.z;
  if (iu >= g.cols || r0 >= g.rows) return;
  const AngleParams& ap = params[theta];
  ColumnEntry ce{};
  if (ap.separable) ce = columns[(size_t)theta * g.cols + iu];
  float prev = weighted_pixel(ap, ce, sino, g, r0, iu, theta);
  const int r1 = min(r0 + kWeightRows, g.rows);
  for (int iv = r0; iv < r1; ++iv) {
    const float next = weighted_pixel(ap, ce, sino, g, iv + 1, iu, theta);
    out[((long long)iv * g.nangles + theta) * g.cols + iu] = make_float2(prev, next);
    prev = next;
  }
}

// Element `row` rows below `col`, rows `rs_bytes` bytes apart: a signed
// 32 x 32 -> 64-bit product (int) or a 64-bit one (long long).
template <typename Offset>
__device__ __forceinline__ const float2* row_at(const float2* col, int row, Offset rs_bytes) {
  return reinterpret_cast<const float2*>(reinterpret_cast<const char*>(col) +
                                         (long long)row * (long long)rs_bytes);
}

// Matched backprojection of separable angles (det_v along z, so b = z) that
// share their in-plane axis a, for kA voxel columns adjacent along a (at
// a-coordinates it0 .. it0 + kA - 1, all on the plane kt of the dominant axis
// d) and the kRun voxels z0 .. z0 + kRun - 1, accumulated into acc.
//
// A detector column iu reaches the voxels of plane kt through
//   h = tent(q_a(iu, kt) - it)           (in-plane weight, one per voxel)
//   V(z) = sum_v tent(q_b(iu, v, kt) - z) W y[v][iu]   (vertical profile)
// and V does not depend on it, so the kA voxels share it: per column and z
// the profile is built once and added with each voxel's h. The columns
// visited are those whose ray passes plane kt within one voxel of any of the
// kA voxels: solve (A0 + A1 u) / (e0 + e1 u) = it0 - 1 and it0 + kA for u.
//
// sinow is the row-pair weighted sinogram (bp_weight_kernel) with kRowPad
// padding rows above and below the detector (rows -kRowPad .. rows + kRowPad
// - 1), so the two-row path reads both rows with one load and without bounds
// tests once its row index is clamped into the padding. Offsets are 32-bit
// unless kWide (padded sinogram of 2^31 pairs or more, or rows 2^31 bytes or
// more apart).
template <int kA, int kRun, bool kWide, bool kFine>
__device__ __forceinline__ void bp_sep_accumulate(const AngleParams* __restrict__ params,
                                                  const ColumnEntry* __restrict__ columns,
                                                  const int* __restrict__ angles, int n_angles,
                                                  const float2* __restrict__ sinow,
                                                  const DeviceGeometry& g, float kt, float it0,
                                                  int z0, float (&acc)[kA][kRun]) {
  using Offset = typename std::conditional<kWide, long long, int>::type;
  const float zt0 = float(z0 - g.oz);
  const Offset rs = Offset(g.nangles) * g.cols;  // row stride
  // row stride in bytes; below 2^31 unless kWide, so a row's address is one
  // 32 x 32 -> 64-bit multiply-add
  const Offset rs_bytes = rs * Offset(sizeof(float2));
  const float2* __restrict__ sinow0 = sinow + (long long)kRowPad * rs;  // row 0
  const float vmin = float(-kRowPad - g.ov), vmax = float(g.rows - g.ov);
  const float4* __restrict__ col4 = reinterpret_cast<const float4*>(columns);
#pragma unroll
  for (int m = 0; m < kA; ++m)
#pragma unroll
    for (int j = 0; j < kRun; ++j) acc[m][j] = 0.0f;

  for (int n = 0; n < n_angles; ++n) {
    const int theta = __ldg(angles + n);
    const AngleParams& ap = params[theta];
    // Only the range needs this solve; the weights below are exact, so fast
    // division is enough.
    const float A0 = fmaf(kt, ap.ma[0], ap.ca[0]);
    const float A1 = fmaf(kt, ap.ma[1], ap.ca[1]);
    const float tl = it0 - 1.0f, th = it0 + float(kA);
    const float u1 = __fdividef(fmaf(tl, ap.e[0], -A0), fmaf(-tl, ap.e[1], A1));
    const float u2 = __fdividef(fmaf(th, ap.e[0], -A0), fmaf(-th, ap.e[1], A1));
    const int iu_lo = max(0, (int)floorf(clamp_coord(fminf(u1, u2))) + 1 + g.ou);
    const int iu_hi = min(g.cols - 1, (int)ceilf(clamp_coord(fmaxf(u1, u2))) - 1 + g.ou);
    const float2* __restrict__ sino_theta = sinow0 + (size_t)theta * g.cols;
    for (int iu = iu_lo; iu <= iu_hi; ++iu) {
      const size_t ci = ((size_t)theta * g.cols + iu) * 2;
      const float4 c0 = __ldg(col4 + ci);      // Xa, ma, P, Q
      const float4 c1 = __ldg(col4 + ci + 1);  // R, S, -, -
      const float qa = fmaf(kt, c0.y, c0.x) - it0;
      float h[kA];
      bool any = false;
#pragma unroll
      for (int m = 0; m < kA; ++m) {
        h[m] = __saturatef(1.0f - fabsf(qa - float(m)));
        any = any || h[m] > 0.0f;
      }
      if (!any) continue;
      // On plane kt, q_b(vt) = B + vt * Sl.
      const float B = fmaf(kt, c0.w, c0.z);
      const float Sl = fmaf(kt, c1.y, c1.x);
      const float inv = __fdividef(1.0f, Sl);
      const float2* __restrict__ col = sino_theta + iu;
      if (fabsf(Sl) >= 1.0f) {
        // Tent half-width 1/|Sl| <= 1 row: only rows floor(v*) and floor(v*)+1.
        // Voxel j's row position vs = (z_j - B) / Sl; row v0's ray passes the
        // plane at t0 = q_b - z_j = v0 Sl + (B - zt0) - j = -Sl (vs - v0), and
        // row v0+1's at t0 + Sl, so |t0 + Sl| = |Sl| - |t0| for the rows the
        // run selects: tent(t0 + Sl) = max(0, 1 - |Sl| + |t0|). Both tents are
        // at most 1 (|t0| >= 0, |t0| < |Sl|), so clamping to [0, 1] is the same
        // max(0, .) and fuses into the add.
        const float C0 = B - zt0;
        const float vs0 = -C0 * inv;  // (zt0 - B) * inv: IEEE subtraction is antisymmetric
        const float vs1 = fmaf(float(kRun - 1), inv, vs0);
        const float c1s = 1.0f - fabsf(Sl);
        const float2* __restrict__ colv = col + Offset(g.ov) * rs;  // row 0 of this column
        // vs is monotone in j: if both ends select rows inside [vmin, vmax]
        // every voxel does, and no clamping is needed (NaN fails the test).
        // Otherwise rows outside [-kRowPad, rows] hold zeros either way:
        // clamping keeps both reads inside the padding (NaN clamps to the low
        // end). Two loops behind a per-column branch (nearly every column is
        // inside) beat one loop with predicated clamps by 14 %.
        const bool inside = fminf(vs0, vs1) >= vmin && fmaxf(vs0, vs1) < vmax + 1.0f;
        // floors by kFloorMagic (no conversion unit); clamping t to the
        // integers [vmin, vmax] clamps its floor (NaN -> vmin)
        if (inside) {
#pragma unroll
          for (int j = 0; j < kRun; ++j) {
            const float f = __fadd_rd(fmaf(float(j), inv, vs0), kFloorMagic);
            const float v0 = f - kFloorMagic;
            const float at0 = fabsf(fmaf(v0, Sl, C0) - float(j));
            const float2 yy = __ldg(row_at(colv, int(__float_as_uint(f) - kFloorBits), rs_bytes));
            const float V = fmaf(__saturatef(1.0f - at0), yy.x, __saturatef(c1s + at0) * yy.y);
#pragma unroll
            for (int m = 0; m < kA; ++m) acc[m][j] = fmaf(h[m], V, acc[m][j]);
          }
        } else {
#pragma unroll
          for (int j = 0; j < kRun; ++j) {
            const float t = fminf(fmaxf(fmaf(float(j), inv, vs0), vmin), vmax);
            const float f = __fadd_rd(t, kFloorMagic);
            const float v0 = f - kFloorMagic;
            const float at0 = fabsf(fmaf(v0, Sl, C0) - float(j));
            const float2 yy = __ldg(row_at(colv, int(__float_as_uint(f) - kFloorBits), rs_bytes));
            const float V = fmaf(__saturatef(1.0f - at0), yy.x, __saturatef(c1s + at0) * yy.y);
#pragma unroll
            for (int m = 0; m < kA; ++m) acc[m][j] = fmaf(h[m], V, acc[m][j]);
          }
        }
      } else if (kFine && fabsf(Sl) >= 0.5f) {
        // (Compiled into the fine-row variant only: the extra path raises the
        // kernel's register pressure.) Rows finer than voxels, |Sl| in
        // [0.5, 1) (a detector supersampled twice, for one): the tent of voxel
        // j (half-width 1/|Sl| <= 2 rows) covers at most four rows, from the
        // first row above its lower end.
        // Two row-pair loads read them; each row is weighted by its exact tent
        // and added in increasing order, as the loop below does, so rows of
        // weight 0 add nothing. The first row is clamped to [vmin, vmax - 1]
        // so both pairs lie in the padded sinogram (rows outside the detector
        // hold zeros; a clamped window still covers the detector rows of the
        // true one; NaN clamps to vmin).
        const float2* __restrict__ colv = col + Offset(g.ov) * rs;  // row 0 of this column
#pragma unroll
        for (int j = 0; j < kRun; ++j) {
          const float Bj = B - (zt0 + float(j));
          float t = fminf((-1.0f - Bj) * inv, (1.0f - Bj) * inv);
          t = fminf(fmaxf(t, vmin - 1.0f), vmax - 2.0f);
          const float f = __fadd_rd(t, kFloorMagic);
          const float v0 = (f - kFloorMagic) + 1.0f;
          const int r0 = int(__float_as_uint(f) - kFloorBits) + 1;
          const float2 y01 = __ldg(row_at(colv, r0, rs_bytes));
          const float2 y23 = __ldg(row_at(colv, r0 + 2, rs_bytes));
          float V = __saturatef(1.0f - fabsf(fmaf(v0, Sl, Bj))) * y01.x;
          V = fmaf(__saturatef(1.0f - fabsf(fmaf(v0 + 1.0f, Sl, Bj))), y01.y, V);
          V = fmaf(__saturatef(1.0f - fabsf(fmaf(v0 + 2.0f, Sl, Bj))), y23.x, V);
          V = fmaf(__saturatef(1.0f - fabsf(fmaf(v0 + 3.0f, Sl, Bj))), y23.y, V);
#pragma unroll
          for (int m = 0; m < kA; ++m) acc[m][j] = fmaf(h[m], V, acc[m][j]);
        }
      } else {
#pragma unroll
        for (int j = 0; j < kRun; ++j) {
          const float Bj = B - (zt0 + float(j));
          const float v1 = (-1.0f - Bj) * inv, v2 = (1.0f - Bj) * inv;
          const int iv_lo = max(0, (int)floorf(clamp_coord(fminf(v1, v2))) + g.ov);
          const int iv_hi = min(g.rows - 1, (int)ceilf(clamp_coord(fmaxf(v1, v2))) + g.ov);
          float V = 0.0f;
          for (int iv = iv_lo; iv <= iv_hi; ++iv) {
            const float w = tent(fmaf(float(iv - g.ov), Sl, Bj));
            V = fmaf(w, __ldg(col + Offset(iv) * rs).x, V);
          }
#pragma unroll
          for (int m = 0; m < kA; ++m) acc[m][j] = fmaf(h[m], V, acc[m][j]);
        }
      }
    }
  }
}

// Epilogues of bp_separable_kernel.
enum BpSepMode {
  kBpSet = 0,        // vol = A^T y
  kBpAdd = 1,        // vol += A^T y
  kBpSirtFirst = 2,  // scratch = this pass's sum (the first of two SIRT passes)
  kBpSirtLast = 3,   // vol += C * (scratch + this pass's sum), or C * sum alone
};

// One pass of the matched backprojection over the separable angles whose
// in-plane axis is x (kAisX: each thread owns kA voxel columns adjacent along
// x on one y) or y (kA columns adjacent along y on one x), with kRun voxels
// along z. The two passes together cover all separable angles; the second
// adds onto the first. In SIRT mode the first pass's sum waits in `scratch`
// so the update x += C * (sum1 + sum2) rounds as the plain recipe's
// vol = sum1; vol += sum2; x += C * vol. Six resident blocks per SM (80
// registers) measured fastest for 2 x 16 voxels per thread: fewer registers
// spill the accumulators, more cut occupancy. A block of 128 threads is kTA
// threads along a times 128 / kTA planes, a-fastest, or plane-fastest (kPF).
template <int kA, int kRun, bool kWide, bool kAisX, int kTA, bool kPF, bool kFine = false>
__device__ __forceinline__ void bp_sep_tile(const AngleParams* __restrict__ params,
                                            const ColumnEntry* __restrict__ columns,
                                            const int* __restrict__ angles, int n_angles,
                                            const float2* __restrict__ sinow,
                                            float* __restrict__ vol, const DeviceGeometry& g,
                                            const float* __restrict__ C,
                                            float* __restrict__ scratch, int mode, int bx, int by,
                                            int bz) {
  constexpr int kTP = kBpX * kBpY / kTA;
  const int t = threadIdx.x;
  const int ta = kPF ? t / kTP : t % kTA;
  const int tp = kPF ? t % kTP : t / kTA;
  // plane-fastest tiles also run their blocks plane-fastest
  const int ba = kPF ? by : bx, bp = kPF ? bx : by;
  const int ia0 = (ba * kTA + ta) * kA;  // first voxel along a
  const int ip = bp * kTP + tp;          // plane
  const int x0 = kAisX ? ia0 : ip;
  const int y0 = kAisX ? ip : ia0;
  const int z0 = bz * kRun;
  if (x0 >= g.nx || y0 >= g.ny) return;
  const float xt = float(x0 - g.ox), yt = float(y0 - g.oy);
  // a = x: the dominant axis is y (kt = y); a = y: it is x.
  const float kt = kAisX ? yt : xt;
  const float it0 = kAisX ? xt : yt;
  float acc[kA][kRun];
  bp_sep_accumulate<kA, kRun, kWide, kFine>(params, columns, angles, n_angles, sinow, g, kt, it0, z0,
                                     acc);
#pragma unroll
  for (int m = 0; m < kA; ++m) {
    const int x = kAisX ? x0 + m : x0, y = kAisX ? y0 : y0 + m;
    if (x >= g.nx || y >= g.ny) continue;
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
      const int z = z0 + j;
      if (z >= g.nz) continue;
      const size_t idx = ((size_t)z * g.ny + y) * g.nx + x;
      if (mode == kBpSet) {
        vol[idx] = acc[m][j];
      } else if (mode == kBpAdd) {
        vol[idx] += acc[m][j];
      } else if (mode == kBpSirtFirst) {
        scratch[idx] = acc[m][j];
      } else {
        const float s = scratch ? __fadd_rn(scratch[idx], acc[m][j]) : acc[m][j];
        vol[idx] = __fadd_rn(vol[idx], __fmul_rn(s, __ldg(C + idx)));
      }
    }
  }
}

// kFine: also the four-row path for detector rows finer than the voxels.
template <int kA, int kRun, bool kWide, bool kAisX, int kMode, int kTA, bool kPF, bool kFine>
__global__ void __launch_bounds__(kBpX* kBpY, 6)
    bp_separable_kernel(const AngleParams* __restrict__ params,
                        const ColumnEntry* __restrict__ columns, const int* __restrict__ angles,
                        int n_angles, const float2* __restrict__ sinow, float* __restrict__ vol,
                        DeviceGeometry g, const float* __restrict__ C,
                        float* __restrict__ scratch) {
  bp_sep_tile<kA, kRun, kWide, kAisX, kTA, kPF, kFine>(params, columns, angles, n_angles, sinow,
                                                       vol, g, C, scratch, kMode, blockIdx.x,
                                                       blockIdx.y, blockIdx.z);
}

// One SIRT pass of many jobs in one launch: block b runs block b - start[j] of
// job j's grid (gx x gy x z blocks, x fastest) with the job's own epilogue
// mode, exactly as bp_separable_kernel would for that job alone. 32-bit
// sinogram offsets only.
template <int kA, int kRun, bool kAisX, int kTA, bool kPF>
__global__ void __launch_bounds__(kBpX* kBpY, 6)
    bp_separable_multi_kernel(const __grid_constant__ BpMulti m) {
  const int j = multi_job_of(m.start, m.n, blockIdx.x);
  const BpMultiJob& J = m.job[j];
  const int local = int(blockIdx.x - m.start[j]);
  const int bx = local % J.gx, r = local / J.gx;
  bp_sep_tile<kA, kRun, false, kAisX, kTA, kPF>(
      J.params, J.columns, J.angles, J.n_angles, reinterpret_cast<const float2*>(J.pairs), J.vol,
      J.g, J.C, J.scratch, J.mode, bx, r % J.gy, r / J.gy);
}

__device__ __forceinline__ float coord(int axis, float z, float y, float x) {
  return axis == 0 ? z : (axis == 1 ? y : x);
}

// Where the weighted value W y of pixel (iv, iu) at angle theta sits in a
// row-pair sinogram: the first half of pair base + iv * s_row + iu * s_col,
// row-major (rows nangles * cols apart) or column-major (rows adjacent).
struct PairView {
  size_t s_row, s_col;
  __device__ __forceinline__ PairView(const DeviceGeometry& g, int zlayout)
      : s_row(zlayout ? 1 : (size_t)g.nangles * g.cols),
        s_col(zlayout ? size_t(g.rows + 2 * kRowPad) : 1) {}
  __device__ __forceinline__ const float2* base(const float2* sinow, const DeviceGeometry& g,
                                                int theta, int zlayout) const {
    return zlayout ? sinow + (size_t)theta * g.cols * s_col + kRowPad
                   : sinow + ((size_t)kRowPad * g.nangles + theta) * g.cols;
  }
};

// The ray of pixel (iu, iv) at one angle, as the forward projector computes it.
__device__ __forceinline__ Ray pixel_ray(const AngleParams& ap,
                                         const ColumnEntry* __restrict__ columns,
                                         const DeviceGeometry& g, int theta, int iu, int iv) {
  const float vt = float(iv - g.ov);
  return ap.separable ? ray_column(columns[(size_t)theta * g.cols + iu], vt)
                      : ray_general(ap, float(iu - g.ou), vt);
}

// Matched-backprojection terms of one voxel (anchored zt, yt, xt) for one
// angle of any geometry, added to acc: project the four corners
// (kt, it -+ 1, jt -+ 1) of the voxel's tent footprint on its plane of the
// dominant axis, and test every pixel of their bounding box with the forward
// projector's ray formula. Rows outer, columns inner.
__device__ __forceinline__ float general_voxel_terms(const AngleParams& ap,
                                                     const ColumnEntry* __restrict__ columns,
                                                     const float2* __restrict__ base,
                                                     const PairView& pv, const DeviceGeometry& g,
                                                     int theta, float zt, float yt, float xt,
                                                     float acc) {
  const float kt = coord(ap.d, zt, yt, xt);
  const float it = coord(ap.a, zt, yt, xt);
  const float jt = coord(ap.b, zt, yt, xt);
  const float nu = fmaf(ap.pu[0], zt, fmaf(ap.pu[1], yt, fmaf(ap.pu[2], xt, ap.pu[3])));
  const float nv = fmaf(ap.pv[0], zt, fmaf(ap.pv[1], yt, fmaf(ap.pv[2], xt, ap.pv[3])));
  const float nw = fmaf(ap.pw[0], zt, fmaf(ap.pw[1], yt, fmaf(ap.pw[2], xt, ap.pw[3])));
  float umin = 3.0e38f, umax = -3.0e38f, vmin = 3.0e38f, vmax = -3.0e38f;
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float da = (c & 1) ? 1.0f : -1.0f, db = (c & 2) ? 1.0f : -1.0f;
    const float cu = fmaf(da, ap.pu[ap.a], fmaf(db, ap.pu[ap.b], nu));
    const float cv = fmaf(da, ap.pv[ap.a], fmaf(db, ap.pv[ap.b], nv));
    const float cw = fmaf(da, ap.pw[ap.a], fmaf(db, ap.pw[ap.b], nw));
    ok = ok && cw > 0.0f;
    const float u = cu / cw, v = cv / cw;
    umin = fminf(umin, u);
    umax = fmaxf(umax, u);
    vmin = fminf(vmin, v);
    vmax = fmaxf(vmax, v);
  }
  if (!ok || !(umin <= umax) || !(vmin <= vmax)) return acc;
  const int iu_lo = max(0, (int)floorf(clamp_coord(umin)) + 1 + g.ou);
  const int iu_hi = min(g.cols - 1, (int)ceilf(clamp_coord(umax)) - 1 + g.ou);
  const int iv_lo = max(0, (int)floorf(clamp_coord(vmin)) + 1 + g.ov);
  const int iv_hi = min(g.rows - 1, (int)ceilf(clamp_coord(vmax)) - 1 + g.ov);
  for (int iv = iv_lo; iv <= iv_hi; ++iv) {
    for (int iu = iu_lo; iu <= iu_hi; ++iu) {
      const Ray r = pixel_ray(ap, columns, g, theta, iu, iv);
      const float wa = tent(fmaf(kt, r.ma, r.Xa) - it);
      const float wb = tent(fmaf(kt, r.mb, r.Xb) - jt);
      const float w = wa * wb;
      if (w > 0.0f) acc = fmaf(w, __ldg(base + iv * pv.s_row + iu * pv.s_col).x, acc);
    }
  }
  return acc;
}

// One thread per voxel; any geometry (the tuning's bp_general = 1).
__global__ void __launch_bounds__(128)
    bp_general_kernel(const AngleParams* __restrict__ params,
                      const ColumnEntry* __restrict__ columns, const int* __restrict__ angles,
                      int n_angles, const float2* __restrict__ sinow, float* __restrict__ vol,
                      DeviceGeometry g, int additive, int zlayout) {
  const int x = blockIdx.x * 32 + threadIdx.x;
  const int y = blockIdx.y * 4 + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= g.nx || y >= g.ny) return;
  const float xt = float(x - g.ox), yt = float(y - g.oy), zt = float(z - g.oz);
  const PairView pv(g, zlayout);
  float acc = 0.0f;
  for (int n = 0; n < n_angles; ++n) {
    const int theta = __ldg(angles + n);
    acc = general_voxel_terms(params[theta], columns, pv.base(sinow, g, theta, zlayout), pv, g,
                              theta, zt, yt, xt, acc);
  }
  float* out = vol + ((size_t)z * g.ny + y) * g.nx + x;
  if (additive)
    *out += acc;
  else
    *out = acc;
}

// ------------------------------------------------- general, staged per box
// The same sums computed by blocks that own a box of voxels and, per angle,
// stage the rays of the detector region the box projects to in shared memory.
// A pixel's ray (a reciprocal and eight multiply-adds) and its weighted value
// are then computed and loaded once per box instead of once per voxel whose
// footprint box contains it. Each voxel bounds its footprint from its centre's
// projection (below) and sums the same candidates, with the same weights, in
// the same order as general_voxel_terms (pixels whose weight is 0 add
// nothing), so both give the same result. Where a region would not fit (a
// detector much finer than the voxels, or a source inside the box's reach), the
// box falls back to general_voxel_terms for that angle.
// Boxes of 16 (z) x 8 (y) x 2 kRunX (x) voxels, kRunX voxels along x per
// thread (the kernel's template argument). kRunX = 8 measured 41.4 ms at
// 256^3 / 360 tilted angles, 4 (boxes of 16 x 8 x 8) 47.0 ms, 16 (80
// registers, 3 blocks per SM) 44.2 ms; the launcher takes 4 where a 16-wide
// box's detector region would not fit the stage (detectors finer than the
// voxels), since those angles would fall back to the per-voxel sums. The
// sinogram layout (kZl) is a template argument too, so that one of the
// stage's two strides is 1 at compile time, and the window shapes of
// gen_window_run's switch (3 x 2, 2 x 2, 3 x 3, 2 x 3 pixels: over 99 % of the
// windows of that scan) are unrolled: 34.6 ms (183.6 ms at 512^3 / 256
// angles, against 227.8 ms with loops over the window at run time; 3 blocks
// per SM instead of 4: 35.3 ms).
constexpr int kGenBoxZ = 16, kGenBoxY = 8;
constexpr int kGenThreads = 256;
constexpr int kGenStage = 2048;                           // staged pixels per angle
constexpr int kGenWindow = 9;  // largest box-wide window (pixels) summed by every voxel
static_assert(kGenWindow < 16, "window shapes are keyed as wu * 16 + wv");

// Detector region of one (box, angle): columns u0 .. u0+nu-1, rows v0 ..
// v0+nv-1; pixel (iu, iv) is staged at (iu - u0) * su + (iv - v0) * sv
// (su = 1 or sv = 1: the sinogram's own order).
// mode 0: no pixel reaches the box; 1: staged, each voxel bounds its own
// footprint; 3: staged, every voxel sums a window of wu x wv pixels from the
// first above (u*, v*) - (hu, hv); 2: per-voxel fallback.
struct GenRegion {
  int u0, v0, nu, nv, su, sv, mode, wu, wv;
  float hu, hv;
};

// Half-extent bound of a voxel footprint's projection, in pixels: a corner
// (+-1 along a and b) of the footprint moves the projection's numerators by
// du (dv) and its denominator by dw, and moves u by (du - u* dw) / (nw + dw),
// at most (S + |u*| E) / (nw - E) with S = |p_a| + |p_b| of that numerator and
// E = |pw_a| + |pw_b| (nw - E is the smallest corner's w). The margin covers
// the rounding of the bound and of the projection: pixels within it of the
// bound have weight 0.
__device__ __forceinline__ float footprint_half(float S, float E, float absu, float rm) {
  return fmaf(fmaf(absu, E, S), rm, fmaf(1e-5f, absu, 1e-2f));
}

// Region of the box [lo, hi] (anchored z, y, x) for one angle, computed by the
// 32 lanes of one warp: lanes 0-7 project the corners of the box widened by
// one voxel (the tent's half-width) along a and b; the projection of the
// box is the convex hull of theirs when every corner lies in front of the
// source (w > 0, an affine function of the position). One pixel of margin on
// each side covers rounding.
__device__ __forceinline__ void gen_region(const AngleParams& ap, const DeviceGeometry& g,
                                           const float (&lo)[3], const float (&hi)[3],
                                           int zlayout, GenRegion* out) {
  const int lane = threadIdx.x & 31;
  float umin = 3.0e38f, umax = -3.0e38f, vmin = 3.0e38f, vmax = -3.0e38f, wmin = 3.0e38f;
  int bad = 0;
  if (lane < 8) {
    float P[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const float e = ax == ap.d ? 0.0f : 1.0f;
      P[ax] = ((lane >> ax) & 1) ? hi[ax] + e : lo[ax] - e;
    }
    const float nu = fmaf(ap.pu[0], P[0], fmaf(ap.pu[1], P[1], fmaf(ap.pu[2], P[2], ap.pu[3])));
    const float nv = fmaf(ap.pv[0], P[0], fmaf(ap.pv[1], P[1], fmaf(ap.pv[2], P[2], ap.pv[3])));
    const float nw = fmaf(ap.pw[0], P[0], fmaf(ap.pw[1], P[1], fmaf(ap.pw[2], P[2], ap.pw[3])));
    const float u = nu / nw, v = nv / nw;
    if (!(nw > 0.0f) || !isfinite(u) || !isfinite(v)) {
      bad = 1;
    } else {
      umin = umax = u;
      vmin = vmax = v;
      wmin = nw;
    }
  }
#pragma unroll
  for (int o = 4; o >= 1; o >>= 1) {  // lanes 0-7 exchange among themselves
    umin = fminf(umin, __shfl_xor_sync(0xffffffffu, umin, o));
    umax = fmaxf(umax, __shfl_xor_sync(0xffffffffu, umax, o));
    vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    wmin = fminf(wmin, __shfl_xor_sync(0xffffffffu, wmin, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if (lane != 0) return;
  GenRegion r{};
  if (bad) {
    r.mode = 2;
  } else {
    const int u0 = max(0, (int)floorf(clamp_coord(umin)) + g.ou);
    const int u1 = min(g.cols - 1, (int)ceilf(clamp_coord(umax)) + g.ou);
    const int v0 = max(0, (int)floorf(clamp_coord(vmin)) + g.ov);
    const int v1 = min(g.rows - 1, (int)ceilf(clamp_coord(vmax)) + g.ov);
    r.u0 = u0;
    r.v0 = v0;
    r.nu = u1 - u0 + 1;
    r.nv = v1 - v0 + 1;
    // staged in the sinogram's own order, so the staging reads are coalesced,
    // with an odd stride between columns (rows) so that the two half-warps,
    // kGenRunX voxels apart along x, read different banks
    const int inner = zlayout ? r.nv : r.nu, outer = zlayout ? r.nu : r.nv;
    const int stride = inner | 1;
    if (r.nu <= 0 || r.nv <= 0)
      r.mode = 0;
    else if ((long long)outer * stride > kGenStage)
      r.mode = 2;
    else
      r.mode = 1;
    r.su = zlayout ? stride : 1;
    r.sv = zlayout ? 1 : stride;
    // One window for the whole box: every voxel centre lies inside the
    // widened box, so its |u*|, |v*| and nw are bounded by the corners' (w is
    // affine, u and v are monotone along lines), and so is its footprint
    // bound. The pixels strictly inside (u* - hu, u* + hu) are at most
    // ceil(2 hu) consecutive ones from floor(u* - hu) + 1.
    const float E = fabsf(ap.pw[ap.a]) + fabsf(ap.pw[ap.b]);
    if (r.mode == 1 && wmin - E > 0.0f) {
      const float rm = 1.0f / (wmin - E);
      r.hu = footprint_half(fabsf(ap.pu[ap.a]) + fabsf(ap.pu[ap.b]), E,
                            fmaxf(fabsf(umin), fabsf(umax)), rm);
      r.hv = footprint_half(fabsf(ap.pv[ap.a]) + fabsf(ap.pv[ap.b]), E,
                            fmaxf(fabsf(vmin), fabsf(vmax)), rm);
      r.wu = (int)ceilf(2.0f * r.hu);
      r.wv = (int)ceilf(2.0f * r.hv);
      if (r.wu >= 1 && r.wv >= 1 && r.wu * r.wv <= kGenWindow && r.wu <= r.nu && r.wv <= r.nv)
        r.mode = 3;
    }
  }
  *out = r;
}

// One thread's kGenRunX voxels (z, y, x0 + m) summed over the box-wide
// window of region R (mode 3) for angle ap. kWu x kWv > 0: the window's shape
// at compile time (loops unrolled, stage offsets hoisted); 0 x 0: R.wu x R.wv
// at run time. kZl: the stage's columns are its strided dimension (column-major
// sinogram; else its rows are). Rows outer, columns inner, as in
// general_voxel_terms, so every form gives the same sums.
template <int kGenRunX, int kZl, int kWu, int kWv>
__device__ __forceinline__ void gen_window_run(const AngleParams& ap, const GenRegion& R,
                                               const DeviceGeometry& g,
                                               const float4* __restrict__ s_ray,
                                               const float* __restrict__ s_val, float zt,
                                               float yt, float xt0, int x0,
                                               float (&acc)[kGenRunX]) {
  const int d = ap.d, a = ap.a;
  const float kt0 = d == 0 ? zt : (d == 1 ? yt : xt0);
  const float it0 = a == 0 ? zt : (a == 1 ? yt : xt0);
  const float jt0 = (d != 0 && a != 0) ? zt : ((d != 1 && a != 1) ? yt : xt0);
  const float dk = d == 2 ? 1.0f : 0.0f, di = a == 2 ? 1.0f : 0.0f;
  const float dj = 1.0f - dk - di;
  const float nu0 = fmaf(ap.pu[0], zt, fmaf(ap.pu[1], yt, fmaf(ap.pu[2], xt0, ap.pu[3])));
  const float nv0 = fmaf(ap.pv[0], zt, fmaf(ap.pv[1], yt, fmaf(ap.pv[2], xt0, ap.pv[3])));
  const float nw0 = fmaf(ap.pw[0], zt, fmaf(ap.pw[1], yt, fmaf(ap.pw[2], xt0, ap.pw[3])));
  const float pu2 = ap.pu[2], pv2 = ap.pv[2], pw2 = ap.pw[2];
  // first pixel above u* - hu, as an index: floor(u* - hu) + 1 + anchor;
  // the window is then moved inside the region if it sticks out (the
  // footprint itself lies inside the region)
  const float ou = float(1 + g.ou) - R.hu, ov = float(1 + g.ov) - R.hv;
  const int u_first = R.u0 + R.nu - R.wu, v_first = R.v0 + R.nv - R.wv;
  const int su = kZl ? R.su : 1, sv = kZl ? 1 : R.sv;
#pragma unroll
  for (int m = 0; m < kGenRunX; ++m) {
    if (x0 + m >= g.nx) break;
    const float fm = float(m);
    const float kt = fmaf(fm, dk, kt0), it = fmaf(fm, di, it0), jt = fmaf(fm, dj, jt0);
    const float rw = __fdividef(1.0f, fmaf(fm, pw2, nw0));
    const float us = fmaf(fm, pu2, nu0) * rw, vs = fmaf(fm, pv2, nv0) * rw;
    const int iu0 = min(max(__float2int_rd(us + ou), R.u0), u_first);
    const int iv0 = min(max(__float2int_rd(vs + ov), R.v0), v_first);
    const int st0 = (iv0 - R.v0) * sv + (iu0 - R.u0) * su;
    float acc_m = acc[m];
    if (kWu > 0) {
#pragma unroll
      for (int r = 0; r < kWv; ++r) {
#pragma unroll
        for (int c = 0; c < kWu; ++c) {
          const int st = st0 + r * sv + c * su;
          const float4 r4 = s_ray[st];
          const float wa = __saturatef(1.0f - fabsf(fmaf(kt, r4.y, r4.x) - it));
          const float wb = __saturatef(1.0f - fabsf(fmaf(kt, r4.w, r4.z) - jt));
          acc_m = fmaf(wa * wb, s_val[st], acc_m);
        }
      }
    } else {
      for (int r = 0; r < R.wv; ++r) {
        for (int c = 0; c < R.wu; ++c) {
          const int st = st0 + r * sv + c * su;
          const float4 r4 = s_ray[st];
          const float wa = __saturatef(1.0f - fabsf(fmaf(kt, r4.y, r4.x) - it));
          const float wb = __saturatef(1.0f - fabsf(fmaf(kt, r4.w, r4.z) - jt));
          acc_m = fmaf(wa * wb, s_val[st], acc_m);
        }
      }
    }
    acc[m] = acc_m;
  }
}

template <int kGenRunX, int kZl>
__global__ void __launch_bounds__(kGenThreads, 4)
    bp_general_box_kernel(const AngleParams* __restrict__ params,
                          const ColumnEntry* __restrict__ columns,
                          const int* __restrict__ angles, int n_angles,
                          const float2* __restrict__ sinow, float* __restrict__ vol,
                          DeviceGeometry g, int additive) {
  constexpr int zlayout = kZl;
  __shared__ float4 s_ray[kGenStage];  // Xa, ma, Xb, mb
  __shared__ float s_val[kGenStage];   // W y
  __shared__ GenRegion s_reg[2];       // regions of angles n and n + 1
  const int tid = threadIdx.x, warp = tid >> 5;
  constexpr int kGenBoxX = 2 * kGenRunX;
  static_assert(kGenBoxZ * kGenBoxY * kGenBoxX / kGenRunX == kGenThreads, "one thread per x run");
  const int bz = blockIdx.z * kGenBoxZ, by = blockIdx.y * kGenBoxY, bx = blockIdx.x * kGenBoxX;
  // this thread's voxels: (z, y, x0 + m), m < kGenRunX
  const int z = bz + (tid & 15), y = by + (tid >> 5), x0 = bx + ((tid >> 4) & 1) * kGenRunX;
  const bool zy_in = z < g.nz && y < g.ny;
  const float zt = float(z - g.oz), yt = float(y - g.oy);
  // the box, clipped to the volume, in anchored coordinates (z, y, x)
  const float lo[3] = {float(bz - g.oz), float(by - g.oy), float(bx - g.ox)};
  const float hi[3] = {float(min(bz + kGenBoxZ, g.nz) - 1 - g.oz),
                       float(min(by + kGenBoxY, g.ny) - 1 - g.oy),
                       float(min(bx + kGenBoxX, g.nx) - 1 - g.ox)};
  const PairView pv(g, zlayout);
  float acc[kGenRunX];
#pragma unroll
  for (int m = 0; m < kGenRunX; ++m) acc[m] = 0.0f;
  if (warp == 0 && n_angles > 0) gen_region(params[__ldg(angles)], g, lo, hi, zlayout, &s_reg[0]);
  __syncthreads();
  const float xt0 = float(x0 - g.ox);
  for (int n = 0; n < n_angles; ++n) {
    const int theta = __ldg(angles + n);
    const AngleParams& ap = params[theta];
    const GenRegion R = s_reg[n & 1];
    const float2* __restrict__ base = pv.base(sinow, g, theta, zlayout);
    if (warp == 0) {
      // the next angle's region, into the slot angle n - 1 used, while the
      // other warps stage this one
      if (n + 1 < n_angles)
        gen_region(params[__ldg(angles + n + 1)], g, lo, hi, zlayout, &s_reg[(n + 1) & 1]);
    } else if (R.mode == 1 || R.mode == 3) {
      // stage the region (warps 1 .. 7): pixel (du, dv) at du * su + dv * sv,
      // walked in storage order
      constexpr int kStagers = kGenThreads - 32;
      const int inner = zlayout ? R.nv : R.nu, total = R.nu * R.nv;
      const int stride = zlayout ? R.su : R.sv;
      const int t0 = tid - 32;
      const int step_q = kStagers / inner, step_r = kStagers % inner;
      int q = t0 / inner, r = t0 % inner;
      for (int t = t0; t < total; t += kStagers) {
        const int iu = R.u0 + (zlayout ? q : r), iv = R.v0 + (zlayout ? r : q);
        const Ray ray = pixel_ray(ap, columns, g, theta, iu, iv);
        const int st = q * stride + r;
        s_ray[st] = make_float4(ray.Xa, ray.ma, ray.Xb, ray.mb);
        s_val[st] = __ldg(base + iv * pv.s_row + iu * pv.s_col).x;
        q += step_q;
        r += step_r;
        if (r >= inner) {
          r -= inner;
          ++q;
        }
      }
    }
    __syncthreads();
    if (zy_in && R.mode == 3) {
      // box-wide window: the same wu x wv candidates for every voxel, so
      // the loops are uniform across the warp and need no per-voxel bound;
      // the common window shapes get fully unrolled sums
      switch (R.wu * 16 + R.wv) {  // wv <= kGenWindow < 16
        case 3 * 16 + 2:
          gen_window_run<kGenRunX, kZl, 3, 2>(ap, R, g, s_ray, s_val, zt, yt, xt0, x0, acc);
          break;
        case 2 * 16 + 2:
          gen_window_run<kGenRunX, kZl, 2, 2>(ap, R, g, s_ray, s_val, zt, yt, xt0, x0, acc);
          break;
        case 3 * 16 + 3:
          gen_window_run<kGenRunX, kZl, 3, 3>(ap, R, g, s_ray, s_val, zt, yt, xt0, x0, acc);
          break;
        case 2 * 16 + 3:
          gen_window_run<kGenRunX, kZl, 2, 3>(ap, R, g, s_ray, s_val, zt, yt, xt0, x0, acc);
          break;
        default:
          gen_window_run<kGenRunX, kZl, 0, 0>(ap, R, g, s_ray, s_val, zt, yt, xt0, x0, acc);
      }
    } else if (zy_in && R.mode == 1) {
      // The thread's voxels run along x, which is one of the angle's axes
      // d, a, b: their (kt, it, jt) step by 1 along that one.
      const int d = ap.d, a = ap.a;
      const float kt0 = d == 0 ? zt : (d == 1 ? yt : xt0);
      const float it0 = a == 0 ? zt : (a == 1 ? yt : xt0);
      const float jt0 = (d != 0 && a != 0) ? zt : ((d != 1 && a != 1) ? yt : xt0);
      const float dk = d == 2 ? 1.0f : 0.0f, di = a == 2 ? 1.0f : 0.0f;
      const float dj = 1.0f - dk - di;
      // footprint bound from the centre's projection (u*, v*) = (nu, nv) / nw
      const float Su = fabsf(ap.pu[a]) + fabsf(ap.pu[ap.b]);
      const float Sv = fabsf(ap.pv[a]) + fabsf(ap.pv[ap.b]);
      const float Ew = fabsf(ap.pw[a]) + fabsf(ap.pw[ap.b]);
      const float nu0 = fmaf(ap.pu[0], zt, fmaf(ap.pu[1], yt, fmaf(ap.pu[2], xt0, ap.pu[3])));
      const float nv0 = fmaf(ap.pv[0], zt, fmaf(ap.pv[1], yt, fmaf(ap.pv[2], xt0, ap.pv[3])));
      const float nw0 = fmaf(ap.pw[0], zt, fmaf(ap.pw[1], yt, fmaf(ap.pw[2], xt0, ap.pw[3])));
      const float pu2 = ap.pu[2], pv2 = ap.pv[2], pw2 = ap.pw[2];
      // pixel index = anchored coordinate + anchor; the first pixel above a
      // bound t is floor(t) + 1, the last below it ceil(t) - 1
      const float lo_u = float(1 + g.ou), hi_u = float(g.ou - 1);
      const float lo_v = float(1 + g.ov), hi_v = float(g.ov - 1);
      const int u_last = R.u0 + R.nu - 1, v_last = R.v0 + R.nv - 1;
#pragma unroll
      for (int m = 0; m < kGenRunX; ++m) {
        if (x0 + m >= g.nx) break;
        const float fm = float(m);
        const float kt = fmaf(fm, dk, kt0), it = fmaf(fm, di, it0), jt = fmaf(fm, dj, jt0);
        const float nu = fmaf(fm, pu2, nu0), nv = fmaf(fm, pv2, nv0), nw = fmaf(fm, pw2, nw0);
        const float rw = __fdividef(1.0f, nw), rm = __fdividef(1.0f, nw - Ew);
        const float us = nu * rw, vs = nv * rw;
        // (rounding of the index computation moves a bound by far less than
        // the margin, so it cannot drop a pixel that has weight)
        const float du = footprint_half(Su, Ew, fabsf(us), rm);
        const float dv = footprint_half(Sv, Ew, fabsf(vs), rm);
        int iu_lo = R.u0, iu_hi = u_last, iv_lo = R.v0, iv_hi = v_last;
        if (nw - Ew > 0.0f) {  // (else: the whole region)
          // float-to-int conversions saturate (NaN -> 0); the region bounds
          // every index
          iu_lo = max(iu_lo, __float2int_rd((us - du) + lo_u));
          iu_hi = min(iu_hi, __float2int_ru((us + du) + hi_u));
          iv_lo = max(iv_lo, __float2int_rd((vs - dv) + lo_v));
          iv_hi = min(iv_hi, __float2int_ru((vs + dv) + hi_v));
        }
        float acc_m = acc[m];
        // stage index of (iv_lo, iu_lo), region-relative (small), then steps
        int st_row = (iv_lo - R.v0) * R.sv + (iu_lo - R.u0) * R.su;
        for (int iv = iv_lo; iv <= iv_hi; ++iv, st_row += R.sv) {
          int st = st_row;
          for (int iu = iu_lo; iu <= iu_hi; ++iu, st += R.su) {
            const float4 r4 = s_ray[st];
            // tent(t) as one saturating add (1 - |t| <= 1; NaN saturates to
            // 0); a weight of 0 adds nothing
            const float wa = __saturatef(1.0f - fabsf(fmaf(kt, r4.y, r4.x) - it));
            const float wb = __saturatef(1.0f - fabsf(fmaf(kt, r4.w, r4.z) - jt));
            acc_m = fmaf(wa * wb, s_val[st], acc_m);
          }
        }
        acc[m] = acc_m;
      }
    } else if (zy_in && R.mode == 2) {
#pragma unroll
      for (int m = 0; m < kGenRunX; ++m)
        if (x0 + m < g.nx)
          acc[m] = general_voxel_terms(ap, columns, base, pv, g, theta, zt, yt,
                                       float(x0 + m - g.ox), acc[m]);
    }
    __syncthreads();  // stage reused and next region visible
  }
  if (!zy_in) return;
#pragma unroll
  for (int m = 0; m < kGenRunX; ++m) {
    if (x0 + m >= g.nx) break;
    float* out = vol + ((size_t)z * g.ny + y) * g.nx + x0 + m;
    if (additive)
      *out += acc[m];
    else
      *out = acc[m];
  }
}

// Matched backprojection of the n general angles at `angles` (device) into
// vol (= or +=), from the row-pair sinogram `pairs` (column-major if zlayout).
// n = 0 with additive = 0 writes zeros. The tuning's bp_general picks the
// box kernel (0) or one thread per voxel (1); both compute the same sums.
void launch_bp_general(const tsgb_projector* p, const int* angles, int n, const float2* pairs,
                       float* vol, bool additive, bool zlayout, cudaStream_t stream) {
  const DeviceGeometry& g = p->g;
  if (p->tuning.bp_general == 1) {
    const dim3 grid((g.nx + 31) / 32, (g.ny + 3) / 4, g.nz);
    bp_general_kernel<<<grid, dim3(32, 4), 0, stream>>>(p->d_params, p->d_columns, angles, n,
                                                        pairs, vol, g, additive ? 1 : 0,
                                                        zlayout ? 1 : 0);
    return;
  }
  const int run = p->gen_box_wide ? 8 : 4, box_x = 2 * run;
  const dim3 grid((g.nx + box_x - 1) / box_x, (g.ny + kGenBoxY - 1) / kGenBoxY,
                  (g.nz + kGenBoxZ - 1) / kGenBoxZ);
  const int add = additive ? 1 : 0;
  if (run == 8 && zlayout)
    bp_general_box_kernel<8, 1><<<grid, kGenThreads, 0, stream>>>(p->d_params, p->d_columns,
                                                                  angles, n, pairs, vol, g, add);
  else if (run == 8)
    bp_general_box_kernel<8, 0><<<grid, kGenThreads, 0, stream>>>(p->d_params, p->d_columns,
                                                                  angles, n, pairs, vol, g, add);
  else if (zlayout)
    bp_general_box_kernel<4, 1><<<grid, kGenThreads, 0, stream>>>(p->d_params, p->d_columns,
                                                                  angles, n, pairs, vol, g, add);
  else
    bp_general_box_kernel<4, 0><<<grid, kGenThreads, 0, stream>>>(p->d_params, p->d_columns,
                                                                  angles, n, pairs, vol, g, add);
}

// Bilinear detector value at anchored (ut, vt), zero outside the detector.
__device__ __forceinline__ float detector_bilinear(const float* __restrict__ base,
                                                   size_t row_stride, const DeviceGeometry& g,
                                                   float ut, float vt) {
  const float fu0 = floorf(ut), fv0 = floorf(vt);
  const float fu = ut - fu0, fv = vt - fv0;
  const int iu = (int)clamp_coord(fu0) + g.ou;
  const int iv = (int)clamp_coord(fv0) + g.ov;
  float v00 = 0.0f, v01 = 0.0f, v10 = 0.0f, v11 = 0.0f;
  const bool u0 = iu >= 0 && iu < g.cols, u1 = iu + 1 >= 0 && iu + 1 < g.cols;
  const bool r0 = iv >= 0 && iv < g.rows, r1 = iv + 1 >= 0 && iv + 1 < g.rows;
  if (r0) {
    const float* row = base + (size_t)iv * row_stride;
    if (u0) v00 = __ldg(row + iu);
    if (u1) v01 = __ldg(row + iu + 1);
  }
  if (r1) {
    const float* row = base + (size_t)(iv + 1) * row_stride;
    if (u0) v10 = __ldg(row + iu);
    if (u1) v11 = __ldg(row + iu + 1);
  }
  const float top = fmaf(fu, v01 - v00, v00);
  const float bot = fmaf(fu, v11 - v10, v10);
  return fmaf(fv, bot - top, top);
}

// Voxel-driven bilinear backprojection of any angle (voxel supersampling
// included). With angle_w (cone beams) the weight is FDK's angle_w[theta] / w^2
// (w = pw . [P, 1], the voxel's depth along the detector normal relative to
// the anchor's) instead of the bilinear backprojector's.
__global__ void __launch_bounds__(kBpX* kBpY)
    bp_bilinear_kernel(const AngleParams* __restrict__ params, const int* __restrict__ angles,
                       int n_angles, const float* __restrict__ sino, float* __restrict__ vol,
                       DeviceGeometry g, int additive, const float* __restrict__ angle_w) {
  const int x = blockIdx.x * kBpX + threadIdx.x;
  const int y = blockIdx.y * kBpY + threadIdx.y;
  const int z0 = blockIdx.z * kRunZBil;
  if (x >= g.nx || y >= g.ny) return;
  const bool cone = g.kind == TSGB_CONE;
  const size_t row_stride = (size_t)g.nangles * g.cols;
  const int ss = g.vox_ss;
  const float inv_ss = 1.0f / float(ss);
  float acc[kRunZBil];
#pragma unroll
  for (int j = 0; j < kRunZBil; ++j) acc[j] = 0.0f;
  for (int n = 0; n < n_angles; ++n) {
    const int theta = __ldg(angles + n);
    const AngleParams& ap = params[theta];
    const float* base = sino + (size_t)theta * g.cols;
    for (int sz = 0; sz < ss; ++sz)
      for (int sy = 0; sy < ss; ++sy)
        for (int sx = 0; sx < ss; ++sx) {
          const float ox = (sx + 0.5f) * inv_ss - 0.5f, oy = (sy + 0.5f) * inv_ss - 0.5f;
          const float oz = (sz + 0.5f) * inv_ss - 0.5f;
          const float xt = float(x - g.ox) + ox, yt = float(y - g.oy) + oy;
#pragma unroll
          for (int j = 0; j < kRunZBil; ++j) {
            const float zt = float(z0 + j - g.oz) + oz;
            const float nu = fmaf(ap.pu[0], zt, fmaf(ap.pu[1], yt, fmaf(ap.pu[2], xt, ap.pu[3])));
            const float nv = fmaf(ap.pv[0], zt, fmaf(ap.pv[1], yt, fmaf(ap.pv[2], xt, ap.pv[3])));
            const float nw = fmaf(ap.pw[0], zt, fmaf(ap.pw[1], yt, fmaf(ap.pw[2], xt, ap.pw[3])));
            const float inw = 1.0f / nw;
            float c = ap.bil_scale;
            if (angle_w) {
              c = nw > 0.0f ? __ldg(angle_w + theta) * inw * inw : 0.0f;
            } else if (cone) {
              const float dz = (zt - ap.src[0]) * g.vs[0], dy = (yt - ap.src[1]) * g.vs[1];
              const float dx = (xt - ap.src[2]) * g.vs[2];
              const float len = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
              c *= len * fabsf(inw * inw * inw);
              if (!(nw > 0.0f)) c = 0.0f;
            }
            const float val = detector_bilinear(base, row_stride, g, nu * inw, nv * inw);
            acc[j] = fmaf(c, val, acc[j]);
          }
        }
  }
  const float norm = inv_ss * inv_ss * inv_ss;
#pragma unroll
  for (int j = 0; j < kRunZBil; ++j) {
    const int z = z0 + j;
    if (z < g.nz) {
      float* out = vol + ((size_t)z * g.ny + y) * g.nx + x;
      if (additive)
        *out += acc[j] * norm;
      else
        *out = acc[j] * norm;
    }
  }
}

// Copy the sinogram into a layout with kRowPad zero rows above and below and
// kColPad zero columns left and right of the detector.
// Detector value at (iv, iu) of angle t, zero outside the detector.
__device__ __forceinline__ float detector_or_zero(const float* __restrict__ sino,
                                                  const DeviceGeometry& g, long long iv,
                                                  long long t, long long iu) {
  if (iu < 0 || iu >= g.cols || iv < 0 || iv >= g.rows) return 0.0f;
  return __ldg(sino + ((size_t)iv * g.nangles + t) * g.cols + iu);
}

// Quad copy of the sinogram for bp_bilinear_z_kernel: element (iv, t, iu) for
// iv in -kRowPad .. rows + kRowPad - 1 and iu in -kColPad .. cols + kColPad - 1
// holds the four taps of a bilinear read, (y[iv][iu], y[iv][iu+1],
// y[iv+1][iu], y[iv+1][iu+1]), zero outside the detector, so one 16-byte
// load serves a voxel.
__global__ void bp_bilinear_prep_kernel(const float* __restrict__ sino, float4* __restrict__ out,
                                        DeviceGeometry g) {
  const long long cp = g.cols + 2 * kColPad, rp = g.rows + 2 * kRowPad;
  const long long total = rp * g.nangles * cp;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long c = idx % cp, rest = idx / cp;
    const long long t = rest % g.nangles, r = rest / g.nangles;
    const long long iu = c - kColPad, iv = r - kRowPad;
    out[idx] = make_float4(detector_or_zero(sino, g, iv, t, iu),
                           detector_or_zero(sino, g, iv, t, iu + 1),
                           detector_or_zero(sino, g, iv + 1, t, iu),
                           detector_or_zero(sino, g, iv + 1, t, iu + 1));
  }
}

// Bilinear backprojection of angles whose projection keeps u and the
// projective denominator constant along z (det_v along z). A thread owns a
// voxel column (x, y) and kRun voxels along z: per angle it projects the
// column once (detector column pair, 1/w, the distance weight's horizontal
// part), then per voxel only steps the detector row and reads one quad.
// sinoq is the quad copy made by bp_bilinear_prep_kernel, so no read needs a
// bounds test once its indices are clamped into the padding (positions
// outside the detector read zeros, as bilinear interpolation with a zero
// border does); a z-run whose rows all lie inside skips the row clamps.
// One voxel's term of the z-flat bilinear backprojection: the quad at row
// floor(vt) of the column (clamped into the zero padding when `clamp`),
// interpolated, times the weight (for cone beams K times the source distance).
template <bool kCone>
__device__ __forceinline__ float bilinear_z_term(const float4* __restrict__ colq, int rs_bytes,
                                                 float vt,
                                                 float vmin, float vmax, bool clamp, float fu,
                                                 float K, float dz, float dxy2, float acc) {
  float fv;
  int row;
  if constexpr (kCone) {
    // Row floor(vt) by kFloorMagic (no conversion unit: the cone weight's
    // rsqrt shares it). Clamping vt to the integers [vmin, vmax] clamps its
    // floor: rows outside read the zero padding (their fraction multiplies
    // zeros; NaN clamps to vmin). Measured 142.6 -> 140.4 ms at 512^3 / 1024;
    // the FDK-weighted variant measured slower with it, so keeps floorf.
    const float t = clamp ? fminf(fmaxf(vt, vmin), vmax) : vt;
    const float f = __fadd_rd(t, kFloorMagic);
    fv = t - (f - kFloorMagic);
    row = int(__float_as_uint(f) - kFloorBits);
  } else {
    float fv0 = floorf(vt);
    fv = vt - fv0;
    if (clamp) fv0 = fminf(fmaxf(fv0, vmin), vmax);  // rows outside read the zero padding
    row = (int)fv0;
  }
  const float4 q = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const char*>(colq) +
                                                       (long long)row * rs_bytes));
  const float top = fmaf(fu, q.y - q.x, q.x);
  const float bot = fmaf(fu, q.w - q.z, q.z);
  const float val = fmaf(fv, bot - top, top);
  float c = K;
  if (kCone) {
    const float l2 = fmaf(dz, dz, dxy2);
    c *= l2 * rsqrtf(l2);
  }
  return fmaf(c, val, acc);
}

// kWeight: kBilParallel, kBilCone (the bilinear backprojector's weights) or
// kBilFdk: FDK's backprojection weight angle_w[theta] / w^2, where w is the
// voxel's depth along the detector normal relative to the volume anchor's
// (the projective denominator pw . [P, 1]).
enum BilWeight { kBilParallel = 0, kBilCone = 1, kBilFdk = 2 };

// A block of 128 threads is kTX voxel columns along x times 128 / kTX along y,
// x-fastest; each thread owns kRun voxels along z.
template <int kRun, int kWeight, int kTX>
__global__ void __launch_bounds__(kBpX* kBpY)
    bp_bilinear_z_kernel(const AngleParams* __restrict__ params, const int* __restrict__ angles,
                         int n_angles, const float4* __restrict__ sinoq, float* __restrict__ vol,
                         DeviceGeometry g, int additive, const float* __restrict__ angle_w) {
  constexpr bool kCone = kWeight == kBilCone;
  constexpr int kTY = kBpX * kBpY / kTX;
  const int x = blockIdx.x * kTX + int(threadIdx.x) % kTX;
  const int y = blockIdx.y * kTY + int(threadIdx.x) / kTX;
  const int z0 = blockIdx.z * kRun;
  if (x >= g.nx || y >= g.ny) return;
  const float xt = float(x - g.ox), yt = float(y - g.oy), zt0 = float(z0 - g.oz);
  const int cp = g.cols + 2 * kColPad;
  const int rs = g.nangles * cp;  // padded row stride (padded copy < 2^31 quads)
  const int rs_bytes = rs * int(sizeof(float4));  // < 2^31 (the plan checks it)
  const float4* __restrict__ base0 = sinoq + kRowPad * rs + kColPad;
  const float umin = float(-kColPad - g.ou), umax = float(g.cols - g.ou);
  const float vmin = float(-kRowPad - g.ov), vmax = float(g.rows - g.ov);
  float acc[kRun];
#pragma unroll
  for (int j = 0; j < kRun; ++j) acc[j] = 0.0f;
  for (int n = 0; n < n_angles; ++n) {
    const int theta = __ldg(angles + n);
    const AngleParams& ap = params[theta];
    const float nw = fmaf(ap.pw[1], yt, fmaf(ap.pw[2], xt, ap.pw[3]));
    if (!(nw > 0.0f)) continue;  // the column lies behind the source
    const float inw = 1.0f / nw;
    const float ut = fmaf(ap.pu[1], yt, fmaf(ap.pu[2], xt, ap.pu[3])) * inw;
    const float fu0 = floorf(ut);
    const float fu = ut - fu0;
    // this column's quads, row 0 (anchored rows count from -ov)
    const float4* __restrict__ colq =
        base0 + theta * cp + ((int)fminf(fmaxf(fu0, umin), umax) + g.ou) + g.ov * rs;
    // vt(j) = (pv0 (zt0 + j) + pv . [y, x, 1]) / w, linear in j
    const float vt0 = fmaf(ap.pv[0], zt0, fmaf(ap.pv[1], yt, fmaf(ap.pv[2], xt, ap.pv[3]))) * inw;
    const float dv = ap.pv[0] * inw;
    float K = ap.bil_scale, dxy2 = 0.0f, dz0 = 0.0f;
    if (kWeight == kBilFdk) K = __ldg(angle_w + theta) * inw * inw;
    if (kCone) {
      K *= inw * inw * inw;
      const float dx = (xt - ap.src[2]) * g.vs[2], dy = (yt - ap.src[1]) * g.vs[1];
      dxy2 = fmaf(dx, dx, dy * dy);
      dz0 = (zt0 - ap.src[0]) * g.vs[0];
    }
    const float vt1 = fmaf(float(kRun - 1), dv, vt0);
    // vt is monotone in j: if both ends read rows inside [vmin, vmax] so does
    // every voxel (NaN fails the test and takes the clamped loop).
    const bool inside = fminf(vt0, vt1) >= vmin && fmaxf(vt0, vt1) < vmax + 1.0f;
    // one loop per case behind a per-column branch (see bp_sep_accumulate)
    if (inside) {
#pragma unroll
      for (int j = 0; j < kRun; ++j)
        acc[j] = bilinear_z_term<kCone>(colq, rs_bytes, fmaf(float(j), dv, vt0), vmin, vmax,
                                        false, fu, K, fmaf(float(j), g.vs[0], dz0), dxy2,
                                        acc[j]);
    } else {
#pragma unroll
      for (int j = 0; j < kRun; ++j)
        acc[j] = bilinear_z_term<kCone>(colq, rs_bytes, fmaf(float(j), dv, vt0), vmin, vmax,
                                        true, fu, K, fmaf(float(j), g.vs[0], dz0), dxy2,
                                        acc[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < kRun; ++j) {
    const int z = z0 + j;
    if (z < g.nz) {
      float* out = vol + ((size_t)z * g.ny + y) * g.nx + x;
      if (additive)
        *out += acc[j];
      else
        *out = acc[j];
    }
  }
}

}  // namespace

namespace {

constexpr int kSepA = 2;  // voxel columns per thread along a (matched)

// Grid of a pass with kTA threads along a, a-fastest or plane-fastest (kPF).
dim3 sep_grid(const DeviceGeometry& g, bool a_is_x, int ta, bool pf) {
  const int tp = kBpX * kBpY / ta;
  const int n_a = a_is_x ? g.nx : g.ny, n_p = a_is_x ? g.ny : g.nx;
  const unsigned ga = (n_a + ta * kSepA - 1) / (ta * kSepA), gp = (n_p + tp - 1) / tp;
  return dim3(pf ? gp : ga, pf ? ga : gp, (g.nz + kRunZ - 1) / kRunZ);
}

// Projectors with rows finer than the voxels (fine_rows) take the fine-row
// variant for plain backprojections with 32-bit offsets; batched SIRT passes
// and 64-bit offsets keep the general row loop for them.
template <bool kWide, bool kAisX, int kMode, int kTA, bool kPF>
void launch_sep_tile(const tsgb_projector* p, const int* angles, int n, const float2* pairs,
                     float* vol, const float* C, float* scratch, cudaStream_t stream) {
  const dim3 grid = sep_grid(p->g, kAisX, kTA, kPF);
  if constexpr (!kWide && (kMode == kBpSet || kMode == kBpAdd)) {
    if (p->fine_rows) {
      bp_separable_kernel<kSepA, kRunZ, kWide, kAisX, kMode, kTA, kPF, true>
          <<<grid, kBpX * kBpY, 0, stream>>>(p->d_params, p->d_columns, angles, n, pairs, vol,
                                             p->g, C, scratch);
      return;
    }
  }
  bp_separable_kernel<kSepA, kRunZ, kWide, kAisX, kMode, kTA, kPF, false>
      <<<grid, kBpX * kBpY, 0, stream>>>(p->d_params, p->d_columns, angles, n, pairs, vol, p->g,
                                         C, scratch);
}

// Thread tiles of the two passes (bit-identical results; measured at 512^3 /
// 1024 angles). a = x: a warp is 8 voxel pairs along x times 4 planes (y); its
// row-pair loads reach about 18 detector columns of rows that adjacent planes
// share, 2.6 % faster than 32 pairs along x (68 columns). a = y: a warp is 32
// planes (x) of one voxel pair along y, plane-fastest, which also keeps the
// stores along x contiguous; tiles with 8 or 16 planes were slower.
constexpr int kTileAx = 8, kTileAy = 4;  // threads along a of the two passes
constexpr bool kPlaneFastAx = false, kPlaneFastAy = true;

template <bool kWide, bool kAisX, int kMode>
void launch_sep_pass_t(const tsgb_projector* p, const int* angles, int n, const float2* pairs,
                       float* vol, const float* C, float* scratch, cudaStream_t stream) {
  if constexpr (kAisX)
    launch_sep_tile<kWide, kAisX, kMode, kTileAx, kPlaneFastAx>(p, angles, n, pairs, vol, C,
                                                                scratch, stream);
  else
    launch_sep_tile<kWide, kAisX, kMode, kTileAy, kPlaneFastAy>(p, angles, n, pairs, vol, C,
                                                                scratch, stream);
}

template <bool kWide, bool kAisX>
void launch_sep_pass_m(const tsgb_projector* p, const int* angles, int n, int mode,
                       const float2* pairs, float* vol, const float* C, float* scratch,
                       cudaStream_t stream) {
  switch (mode) {
    case kBpSet:
      launch_sep_pass_t<kWide, kAisX, kBpSet>(p, angles, n, pairs, vol, C, scratch, stream);
      break;
    case kBpAdd:
      launch_sep_pass_t<kWide, kAisX, kBpAdd>(p, angles, n, pairs, vol, C, scratch, stream);
      break;
    case kBpSirtFirst:
      launch_sep_pass_t<kWide, kAisX, kBpSirtFirst>(p, angles, n, pairs, vol, C, scratch, stream);
      break;
    default:
      launch_sep_pass_t<kWide, kAisX, kBpSirtLast>(p, angles, n, pairs, vol, C, scratch, stream);
  }
}

// One pass of the separable matched backprojection over the n angle ids at
// `angles` (device), all with in-plane axis x (a_is_x) or all with y.
// 32-bit offsets need fewer than 2^31 padded pairs and a row stride below
// 2^31 bytes
bool sep_wide(const DeviceGeometry& g) {
  const size_t rs = (size_t)g.nangles * g.cols;
  return (size_t)(g.rows + 2 * kRowPad) * rs >= (size_t(1) << 31) ||
         rs * sizeof(float2) >= (size_t(1) << 31);
}

void launch_sep_pass(const tsgb_projector* p, bool a_is_x, const int* angles, int n, int mode,
                     const float2* pairs, float* vol, const float* C, float* scratch,
                     cudaStream_t stream) {
  const bool wide = sep_wide(p->g);
  if (wide && a_is_x)
    launch_sep_pass_m<true, true>(p, angles, n, mode, pairs, vol, C, scratch, stream);
  else if (wide)
    launch_sep_pass_m<true, false>(p, angles, n, mode, pairs, vol, C, scratch, stream);
  else if (a_is_x)
    launch_sep_pass_m<false, true>(p, angles, n, mode, pairs, vol, C, scratch, stream);
  else
    launch_sep_pass_m<false, false>(p, angles, n, mode, pairs, vol, C, scratch, stream);
}

// Row-major row-pair weighted sinogram of angles [angle_begin, angle_end)
// into `pairs` (bp_weight_kernel), and the padding rows it does not write
// zeroed: -kRowPad .. -2 and rows .. rows + kRowPad - 1.
void launch_bp_weight_rows(const tsgb_projector* p, const float* sino, float2* pairs,
                           int angle_begin, int angle_end, cudaStream_t stream) {
  const DeviceGeometry& g = p->g;
  const size_t rs = (size_t)g.nangles * g.cols;  // elements between rows
  const dim3 block(32, 8);
  for (int a0 = angle_begin; a0 < angle_end; a0 += 65535) {
    const int n = angle_end - a0 < 65535 ? angle_end - a0 : 65535;
    const dim3 grid((g.cols + 31) / 32, (g.rows + 1 + 8 * kWeightRows - 1) / (8 * kWeightRows),
                    n);
    // offset the angle through the pointers: rows are strided by nangles*cols
    bp_weight_kernel<<<grid, block, 0, stream>>>(p->d_params + a0, p->d_columns + (size_t)a0 * g.cols,
                                                 sino + (size_t)a0 * g.cols,
                                                 pairs + kRowPad * rs + (size_t)a0 * g.cols, g);
  }
  cudaMemsetAsync(pairs, 0, (kRowPad - 1) * rs * sizeof(float2), stream);
  cudaMemsetAsync(pairs + (kRowPad + g.rows) * rs, 0, kRowPad * rs * sizeof(float2), stream);
}

// Entries of host_list[lo, hi) (angle ids in increasing order) that lie in
// [a0, a1): offset into the list and count.
void angle_sub_range(const std::vector<int>& host_list, int lo, int hi, int a0, int a1, int& off,
                     int& n) {
  const auto b = host_list.begin();
  const auto first = std::lower_bound(b + lo, b + hi, a0);
  const auto last = std::lower_bound(first, b + hi, a1);
  off = int(first - b);
  n = int(last - first);
}

}  // namespace

int launch_bp_matched(const tsgb_projector* p, float* vol, const float* sino, bool additive,
                      float* workspace, void* stream_, int angle_begin, int angle_end) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const DeviceGeometry& g = p->g;
  if (angle_end < 0) angle_end = g.nangles;
  // the angles of [angle_begin, angle_end) in each of the three angle lists
  int off_x, n_ax, off_y, n_ay, off_g, n_g;
  angle_sub_range(p->host_sep_angles, 0, p->n_sep_ax, angle_begin, angle_end, off_x, n_ax);
  angle_sub_range(p->host_sep_angles, p->n_sep_ax, p->n_separable_bp, angle_begin, angle_end,
                  off_y, n_ay);
  angle_sub_range(p->host_gen_angles, 0, p->n_general_bp, angle_begin, angle_end, off_g, n_g);
  float2* pairs = reinterpret_cast<float2*>(workspace);
  if (bp_uses_zlane(p)) {
    // column-major weighted sinogram, z-lane passes into the [y][x][z]
    // scratch that follows it, then the caller's volume
    launch_bp_weight_z(p, sino, workspace, angle_begin, angle_end, stream);
    float* volt = reinterpret_cast<float*>(reinterpret_cast<char*>(workspace) + bp_pairs_bytes(g));
    const bool written = launch_bp_zlane_separable(p, off_x, n_ax, off_y, n_ay, workspace, volt, vol,
                                                   additive ? 1 : 0, nullptr, stream);
    if (n_g > 0 || (!written && !additive))
      launch_bp_general(p, p->d_gen_angles + off_g, n_g, pairs, vol, additive || written, true,
                        stream);
    return int(cudaGetLastError());
  }
  launch_bp_weight_rows(p, sino, pairs, angle_begin, angle_end, stream);
  if (n_ax > 0)
    launch_sep_pass(p, true, p->d_sep_angles + off_x, n_ax, additive ? kBpAdd : kBpSet, pairs,
                    vol, nullptr, nullptr, stream);
  if (n_ay > 0)
    launch_sep_pass(p, false, p->d_sep_angles + off_y, n_ay,
                    (additive || n_ax > 0) ? kBpAdd : kBpSet, pairs, vol, nullptr, nullptr, stream);
  const bool written = n_ax + n_ay > 0;
  if (n_g > 0 || (!written && !additive))
    launch_bp_general(p, p->d_gen_angles + off_g, n_g, pairs, vol, additive || written, false,
                      stream);
  return int(cudaGetLastError());
}

namespace {

// vol += C * s elementwise, rounded as the plain recipe's x_tmp *= C; x += x_tmp.
__global__ void sirt_update_kernel(float* __restrict__ vol, const float* __restrict__ C,
                                   const float* __restrict__ s, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    vol[i] = __fadd_rn(vol[i], __fmul_rn(__ldg(s + i), __ldg(C + i)));
}

}  // namespace

int launch_bp_sirt(const tsgb_projector* p, float* vol, const float* C, const float* res,
                   float* scratch, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const float2* pairs = reinterpret_cast<const float2*>(res);
  const int n_ax = p->n_sep_ax, n_ay = p->n_separable_bp - p->n_sep_ax;
  const DeviceGeometry& g = p->g;
  if (p->n_general_bp > 0) {
    // Angles outside the separable backprojector (tilted detectors): the whole
    // backprojection goes into a sum volume as launch_bp_matched computes it
    // (separable passes, then the general kernel adding), and the update is a
    // separate element-wise pass. scratch holds the sum, then the z-lane
    // kernel's own scratch (the forward workspace fits both).
    float* vsum = scratch;
    bool written = false;
    if (bp_uses_zlane(p)) {
      float* volt = reinterpret_cast<float*>(reinterpret_cast<char*>(scratch) + bp_volume_bytes(g));
      written = launch_bp_zlane_separable(p, 0, n_ax, n_ax, n_ay, res, volt, vsum, 0, nullptr,
                                          stream);
    } else {
      if (n_ax > 0)
        launch_sep_pass(p, true, p->d_sep_angles, n_ax, kBpSet, pairs, vsum, nullptr, nullptr,
                        stream);
      if (n_ay > 0)
        launch_sep_pass(p, false, p->d_sep_angles + n_ax, n_ay, n_ax > 0 ? kBpAdd : kBpSet, pairs,
                        vsum, nullptr, nullptr, stream);
      written = n_ax + n_ay > 0;
    }
    launch_bp_general(p, p->d_gen_angles, p->n_general_bp, pairs, vsum, written,
                      bp_uses_zlane(p), stream);
    const long long n = (long long)g.nz * g.ny * g.nx;
    const long long blocks = (n + 255) / 256;
    sirt_update_kernel<<<int(blocks < 152LL * 32 ? blocks : 152LL * 32), 256, 0, stream>>>(
        vol, C, vsum, n);
    return int(cudaGetLastError());
  }
  if (bp_uses_zlane(p)) {
    // the residual is column-major; scratch holds the [y][x][z] sum
    launch_bp_zlane_separable(p, 0, n_ax, n_ax, n_ay, res, scratch, vol, 2, C, stream);
    return int(cudaGetLastError());
  }
  const int* ax = p->d_sep_angles;
  const int* ay = p->d_sep_angles + n_ax;
  if (n_ax > 0 && n_ay > 0) {
    launch_sep_pass(p, true, ax, n_ax, kBpSirtFirst, pairs, vol, C, scratch, stream);
    launch_sep_pass(p, false, ay, n_ay, kBpSirtLast, pairs, vol, C, scratch, stream);
  } else if (n_ax > 0) {
    launch_sep_pass(p, true, ax, n_ax, kBpSirtLast, pairs, vol, C, nullptr, stream);
  } else if (n_ay > 0) {
    launch_sep_pass(p, false, ay, n_ay, kBpSirtLast, pairs, vol, C, nullptr, stream);
  }
  return int(cudaGetLastError());
}

long long bp_sep_blocks(const tsgb_projector* p, bool a_is_x, int* gx, int* gy) {
  if (sep_wide(p->g)) return -1;
  const dim3 grid = a_is_x ? sep_grid(p->g, true, kTileAx, kPlaneFastAx)
                           : sep_grid(p->g, false, kTileAy, kPlaneFastAy);
  *gx = int(grid.x);
  *gy = int(grid.y);
  return (long long)grid.x * grid.y * grid.z;
}

int launch_bp_sep_multi(const BpMulti& m, bool a_is_x, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const long long blocks = m.start[m.n];
  if (blocks <= 0) return int(cudaGetLastError());
  if (a_is_x)
    bp_separable_multi_kernel<kSepA, kRunZ, true, kTileAx, kPlaneFastAx>
        <<<unsigned(blocks), kBpX * kBpY, 0, stream>>>(m);
  else
    bp_separable_multi_kernel<kSepA, kRunZ, false, kTileAy, kPlaneFastAy>
        <<<unsigned(blocks), kBpX * kBpY, 0, stream>>>(m);
  return int(cudaGetLastError());
}

bool bp_batch_multi_eligible(const tsgb_projector* p) {
  int gx = 0, gy = 0;
  return !p->fine && !bp_uses_zlane(p) && !p->fine_rows && p->n_general_bp == 0 &&
         p->n_separable_bp > 0 && bp_sep_blocks(p, true, &gx, &gy) >= 0 &&
         bp_sep_blocks(p, false, &gx, &gy) >= 0;
}

int launch_bp_matched_batch(const tsgb_projector* p, float* vol, const float* sino, int64_t n,
                            bool additive, char* workspace, int64_t item_bytes, int group,
                            void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const DeviceGeometry& g = p->g;
  const size_t vol_elems = size_t(g.nz) * g.ny * g.nx;
  const size_t sino_elems = size_t(g.rows) * g.nangles * g.cols;
  const int n_ax = p->n_sep_ax, n_ay = p->n_separable_bp - p->n_sep_ax;
  for (int64_t i0 = 0; i0 < n; i0 += group) {
    const int m = int(std::min<int64_t>(group, n - i0));
    for (int k = 0; k < m; ++k)
      launch_bp_weight_rows(p, sino + (i0 + k) * sino_elems,
                            reinterpret_cast<float2*>(workspace + k * item_bytes), 0, g.nangles,
                            stream);
    // the pass along x sets (or adds), the pass along y adds onto it
    for (int pass = 0; pass < 2; ++pass) {
      const bool a_is_x = pass == 0;
      const int n_pass = a_is_x ? n_ax : n_ay;
      if (n_pass == 0) continue;
      BpMulti bm{};
      for (int k = 0; k < m; ++k) {
        BpMultiJob& J = bm.job[k];
        J.params = p->d_params;
        J.columns = p->d_columns;
        J.angles = p->d_sep_angles + (a_is_x ? 0 : n_ax);
        J.n_angles = n_pass;
        J.pairs = reinterpret_cast<const float*>(workspace + k * item_bytes);
        J.vol = vol + (i0 + k) * vol_elems;
        J.C = nullptr;
        J.scratch = nullptr;
        J.mode = (additive || (!a_is_x && n_ax > 0)) ? kBpAdd : kBpSet;
        J.g = g;
        bm.start[k + 1] = bm.start[k] + bp_sep_blocks(p, a_is_x, &J.gx, &J.gy);
      }
      bm.n = m;
      const int rc = launch_bp_sep_multi(bm, a_is_x, stream);
      if (rc != 0) return rc;
    }
  }
  return int(cudaGetLastError());
}

namespace {

template <int kWeight, int kTX>
void launch_bil_z_tile(const tsgb_projector* p, const float4* quads, float* vol, bool additive,
                       const float* angle_w, cudaStream_t stream) {
  const DeviceGeometry& g = p->g;
  constexpr int kTY = kBpX * kBpY / kTX;
  const dim3 grid((g.nx + kTX - 1) / kTX, (g.ny + kTY - 1) / kTY, (g.nz + kRunZ - 1) / kRunZ);
  bp_bilinear_z_kernel<kRunZ, kWeight, kTX><<<grid, kBpX * kBpY, 0, stream>>>(
      p->d_params, p->d_bil_fast, p->n_bil_fast, quads, vol, g, additive ? 1 : 0, angle_w);
}

// A warp of the z-flat bilinear kernel is 8 voxel columns along x times 4
// along y: its quad loads reach fewer detector columns and rows than 32
// columns along x (153 -> 143 ms at 512^3 / 1024 angles; 4 x 8 measured the
// same, 2 x 16 slower), and its stores still fill 32-byte sectors.
template <int kWeight>
void launch_bil_z(const tsgb_projector* p, const float4* quads, float* vol, bool additive,
                  const float* angle_w, cudaStream_t stream) {
  launch_bil_z_tile<kWeight, 8>(p, quads, vol, additive, angle_w, stream);
}

}  // namespace

int launch_bp_bilinear(const tsgb_projector* p, float* vol, const float* sino, bool additive,
                       float* workspace, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const DeviceGeometry& g = p->g;
  const dim3 block(kBpX, kBpY);
  bool written = false;
  if (p->n_bil_fast > 0) {
    const long long total = (long long)(g.rows + 2 * kRowPad) * g.nangles * (g.cols + 2 * kColPad);
    const long long blocks = (total + 255) / 256;
    float4* quads = reinterpret_cast<float4*>(workspace);
    bp_bilinear_prep_kernel<<<int(blocks < 152LL * 64 ? blocks : 152LL * 64), 256, 0, stream>>>(
        sino, quads, g);
    if (g.kind == TSGB_CONE)
      launch_bil_z<kBilCone>(p, quads, vol, additive, nullptr, stream);
    else
      launch_bil_z<kBilParallel>(p, quads, vol, additive, nullptr, stream);
    written = true;
  }
  if (p->n_bil_slow > 0 || !written) {
    const dim3 grid((g.nx + kBpX - 1) / kBpX, (g.ny + kBpY - 1) / kBpY,
                    (g.nz + kRunZBil - 1) / kRunZBil);
    bp_bilinear_kernel<<<grid, block, 0, stream>>>(p->d_params, p->d_bil_slow, p->n_bil_slow, sino,
                                                   vol, g, (additive || written) ? 1 : 0, nullptr);
  }
  return int(cudaGetLastError());
}

int launch_bp_fdk(const tsgb_projector* p, float* vol, const float* sino, const float* angle_w,
                  bool additive, float* workspace, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const DeviceGeometry& g = p->g;
  bool written = false;
  if (p->n_bil_fast > 0) {
    const long long total = (long long)(g.rows + 2 * kRowPad) * g.nangles * (g.cols + 2 * kColPad);
    const long long blocks = (total + 255) / 256;
    float4* quads = reinterpret_cast<float4*>(workspace);
    bp_bilinear_prep_kernel<<<int(blocks < 152LL * 64 ? blocks : 152LL * 64), 256, 0, stream>>>(
        sino, quads, g);
    launch_bil_z<kBilFdk>(p, quads, vol, additive, angle_w, stream);
    written = true;
  }
  if (p->n_bil_slow > 0 || !written) {
    // angles whose projection depends on z (tilted detectors, rotated scans)
    const dim3 grid((g.nx + kBpX - 1) / kBpX, (g.ny + kBpY - 1) / kBpY,
                    (g.nz + kRunZBil - 1) / kRunZBil);
    bp_bilinear_kernel<<<grid, dim3(kBpX, kBpY), 0, stream>>>(
        p->d_params, p->d_bil_slow, p->n_bil_slow, sino, vol, g, (additive || written) ? 1 : 0,
        angle_w);
  }
  return int(cudaGetLastError());
}

}  // namespace tsgb
