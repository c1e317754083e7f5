// Matched backprojection of separable angles with z-lane warps.
//
// The exact transpose of fp_ray_kernel for angles whose det_v runs along z
// (b = z: circular and helical cone and parallel scans), as bp_separable_kernel
// computes it, with the work laid out differently:
//
//  * The weighted sinogram is stored column-major: element (theta, iu, r) holds
//    the row pair (W y[v], W y[v+1]) of detector row v = r - kRowPad, rows
//    fastest (bp_weight_z_kernel). Padding pairs (v = -2, rows, rows + 1) and
//    the halves that fall off the detector are zero.
//  * A warp owns kX voxels along the in-plane axis a on one plane of the
//    dominant axis d, and 32 x kRun voxels along z: lane l holds z0 + l + 32 j
//    for j < kRun. On a plane, which detector columns reach a voxel and with
//    what in-plane weight depends only on its a-coordinate, so all 32 lanes
//    walk the same columns: the column loop is uniform (no divergence), and
//    each column's vertical profile V(z) is built once for the whole window
//    (kX + 1 voxel widths of columns per kX voxels, against 3 per 2 when two
//    voxels share a thread). The lanes' row-pair loads of one column fall on
//    about 23 consecutive rows: one or two 128-byte lines per load.
//  * A column whose ray crosses the plane at q_a (window coordinates, floor f0,
//    fraction fa) adds (1 - fa) V to voxel f0 and fa V to voxel f0 + 1 (the
//    tents of the two voxels it lies between); a uniform branch on f0 picks the
//    accumulator registers.
//  * Results go to a z-fastest scratch volume [y][x][z] (both passes, the
//    second adding), so every store is a coalesced 128-byte run; one tiled
//    transpose (bp_zlane_out_kernel) then writes the caller's [z][y][x] volume,
//    setting, adding or applying the SIRT update.
//
// Arithmetic per (column, voxel) is bp_separable_kernel's: the two row tents
// of the fast path (|slope| >= 1 rows per voxel) as saturating adds from the
// exact row position, and the general row loop otherwise. Only the order in
// which each voxel's terms are summed differs (per angle, columns in order).
// Floors and float-to-int conversions of the inner loop avoid the conversion
// unit (see kFloorMagic), which a 512^3 profile showed half busy otherwise.
#include <cuda_runtime.h>

#include <algorithm>

#include "device_common.cuh"

namespace tsgb {
namespace {

constexpr float kMaxSlopeZ = 64.0f;  // must match fp.cu

// W * y of pixel (iv, iu) at angle theta, 0 off the detector and for rays the
// forward projector does not sample.
__device__ __forceinline__ float weighted_pixel_z(const AngleParams& ap, const ColumnEntry& ce,
                                                  const float* __restrict__ sino,
                                                  const DeviceGeometry& g, int iv, int iu,
                                                  int theta) {
  if (iv < 0 || iv >= g.rows || iu >= g.cols) return 0.0f;
  const float vt = float(iv - g.ov);
  const Ray r = ap.separable ? ray_column(ce, vt) : ray_general(ap, float(iu - g.ou), vt);
  float w = 0.0f;
  if (finite_ray(r) && fabsf(r.ma) <= kMaxSlopeZ && fabsf(r.mb) <= kMaxSlopeZ) w = ray_step(ap, r);
  return w * __ldg(sino + ((size_t)iv * g.nangles + theta) * g.cols + iu);
}

// Column-major row-pair weighted sinogram. A block of 32 x 8 threads covers
// 32 detector columns x 32 padded pair rows of one angle: it computes the 33
// rows of W y it needs into shared memory (reads along u, coalesced), then
// writes the pairs along the rows (coalesced). Every padded pair is written,
// so the buffer needs no clearing. `out` points at the angle range's first
// column; blockIdx.z counts angles from `theta0`.
__global__ void __launch_bounds__(256)
    bp_weight_z_kernel(const AngleParams* __restrict__ params,
                       const ColumnEntry* __restrict__ columns, const float* __restrict__ sino,
                       float2* __restrict__ out, DeviceGeometry g, int theta0) {
  __shared__ float s[33][33];  // [row][column]
  const int theta = theta0 + blockIdx.z;
  const int iu0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  const int RP = g.rows + 2 * kRowPad;
  const AngleParams& ap = params[theta];
  {
    const int iu = iu0 + threadIdx.x;
    ColumnEntry ce{};
    if (ap.separable && iu < g.cols) ce = columns[(size_t)theta * g.cols + iu];
    for (int k = threadIdx.y; k < 33; k += 8)
      s[k][threadIdx.x] = weighted_pixel_z(ap, ce, sino, g, r0 + k - kRowPad, iu, theta);
  }
  __syncthreads();
  const int r = r0 + threadIdx.x;
  if (r >= RP) return;
  for (int c = threadIdx.y; c < 32; c += 8) {
    const int iu = iu0 + c;
    if (iu >= g.cols) break;
    out[((size_t)blockIdx.z * g.cols + iu) * RP + r] =
        make_float2(s[threadIdx.x][c], s[threadIdx.x + 1][c]);
  }
}

// Window accumulation: a column between voxels f0 and f0 + 1 of the window
// (f0 in -1 .. kX - 1) adds (1 - fa) V(z) to voxel f0 and fa V(z) to voxel
// f0 + 1, V(z) = profile(j) for the lane's voxel z0 + 32 j. The uniform branch
// on f0 sits outside the z loop, so each profile value goes straight into the
// two accumulators it feeds.
template <int kX, int kRun, int kM, typename F>
__device__ __forceinline__ void window_apply(float (&acc)[kX][kRun], const F& profile, float wl,
                                             float wr) {
#pragma unroll
  for (int j = 0; j < kRun; ++j) {
    const float V = profile(j);
    if constexpr (kM >= 0) acc[kM][j] = fmaf(wl, V, acc[kM][j]);
    if constexpr (kM + 1 < kX) acc[kM + 1][j] = fmaf(wr, V, acc[kM + 1][j]);
  }
}

template <int kX, int kRun, int kM, typename F>
__device__ __forceinline__ void window_dispatch(float (&acc)[kX][kRun], int f0, const F& profile,
                                                float wl, float wr) {
  if constexpr (kM < kX) {
    if (f0 == kM)
      window_apply<kX, kRun, kM>(acc, profile, wl, wr);
    else
      window_dispatch<kX, kRun, kM + 1>(acc, f0, profile, wl, wr);
  }
}

// One pass over the separable angles whose in-plane axis is x (kAisX: planes
// are y) or y (planes are x). Block: kPlanes warps on adjacent planes, same
// window and z range. blockIdx.x = window * plane_blocks + plane block,
// blockIdx.y = z range. volt is the [y][x][z] scratch volume; kAdd: add to it.
// The next column's table entry is loaded while the current one is processed.
template <int kX, int kRun, int kPlanes, int kMinBlocks, bool kAisX, bool kAdd>
__global__ void __launch_bounds__(32 * kPlanes, kMinBlocks)
    bp_zlane_kernel(const AngleParams* __restrict__ params,
                    const ColumnEntry* __restrict__ columns, const int* __restrict__ angles,
                    int n_angles, const float2* __restrict__ sinoz, float* __restrict__ volt,
                    DeviceGeometry g, int plane_blocks) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n_p = kAisX ? g.ny : g.nx, n_a = kAisX ? g.nx : g.ny;
  const int pb = int(blockIdx.x % unsigned(plane_blocks));
  const int wb = int(blockIdx.x / unsigned(plane_blocks));
  const int ip = pb * kPlanes + w;  // plane (along d)
  const int i0 = wb * kX;           // window start (along a)
  if (ip >= n_p) return;            // whole warp
  const int z0 = blockIdx.y * (32 * kRun) + lane;
  const float kt = float(ip - (kAisX ? g.oy : g.ox));
  const float i0t = float(i0 - (kAisX ? g.ox : g.oy));
  const float zt = float(z0 - g.oz);
  const int RP = g.rows + 2 * kRowPad;
  const float vmin = float(-kRowPad - g.ov), vmax = float(g.rows - g.ov);
  float acc[kX][kRun];
#pragma unroll
  for (int m = 0; m < kX; ++m)
#pragma unroll
    for (int j = 0; j < kRun; ++j) acc[m][j] = 0.0f;
  const float4* __restrict__ col4 = reinterpret_cast<const float4*>(columns);

  for (int n = 0; n < n_angles; ++n) {
    const int theta = __ldg(angles + n);
    const AngleParams& ap = params[theta];
    // detector columns whose ray crosses this plane within (i0 - 1, i0 + kX):
    // q_a(u) = (A0 + A1 u) / (e0 + e1 u); only the range uses this solve
    const float A0 = fmaf(kt, ap.ma[0], ap.ca[0]);
    const float A1 = fmaf(kt, ap.ma[1], ap.ca[1]);
    const float tl = i0t - 1.0f, th = i0t + float(kX);
    const float u1 = __fdividef(fmaf(tl, ap.e[0], -A0), fmaf(-tl, ap.e[1], A1));
    const float u2 = __fdividef(fmaf(th, ap.e[0], -A0), fmaf(-th, ap.e[1], A1));
    const int iu_lo = max(0, (int)floorf(clamp_coord(fminf(u1, u2))) + 1 + g.ou);
    const int iu_hi = min(g.cols - 1, (int)ceilf(clamp_coord(fmaxf(u1, u2))) - 1 + g.ou);
    // anchored row 0 of this angle's first column
    const float2* __restrict__ sth = sinoz + (size_t)theta * g.cols * RP + (kRowPad + g.ov);
    // column entries: Xa, ma, P, Q | R, S, -, -
    const float4* __restrict__ cth = col4 + (size_t)theta * g.cols * 2;
    float4 n0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), n1 = n0;
    if (iu_lo <= iu_hi) {
      n0 = __ldg(cth + 2 * iu_lo);
      n1 = __ldg(cth + 2 * iu_lo + 1);
    }
    for (int iu = iu_lo; iu <= iu_hi; ++iu) {
      const float4 c0 = n0, c1 = n1;
      if (iu < iu_hi) {
        n0 = __ldg(cth + 2 * (iu + 1));
        n1 = __ldg(cth + 2 * (iu + 1) + 1);
      }
      const float qa = fmaf(kt, c0.y, c0.x) - i0t;
      if (!(qa > -1.0f && qa < float(kX))) continue;  // (uniform; NaN skips)
      const float fq = __fadd_rd(qa, kFloorMagic);
      const float fa = qa - (fq - kFloorMagic);
      const int f0 = int(__float_as_uint(fq) - kFloorBits);
      // On this plane, q_b(vt) = B + vt * Sl; lane z's rows lie near (z - B) / Sl.
      const float B = fmaf(kt, c0.w, c0.z);
      const float Sl = fmaf(kt, c1.y, c1.x);
      const float inv = __fdividef(1.0f, Sl);
      const float2* __restrict__ col = sth + (size_t)iu * RP;
      const float C0 = B - zt;
      const float wl = 1.0f - fa;
      if (fabsf(Sl) >= 1.0f) {
        // Row pair v0 = floor((z - B) / Sl) and v0 + 1 (tent half-width
        // 1/|Sl| <= 1 row). For voxel z = zt + 32 j: row v0's ray crosses the
        // plane at t0 = v0 Sl + C0 - 32 j from it, row v0+1's at t0 + Sl,
        // so the tents are max(0, 1 - |t0|) and max(0, 1 - |Sl| + |t0|)
        // (both at most 1: saturating adds).
        const float vs0 = -C0 * inv;
        const float dv = 32.0f * inv;
        const float vs1 = fmaf(float(kRun - 1), dv, vs0);
        const float c1s = 1.0f - fabsf(Sl);
        // rows are monotone in j: both ends inside [vmin, vmax] => every row
        // is (NaN fails and takes the clamped loop, which keeps every read
        // inside the zero padding)
        const bool inside = fminf(vs0, vs1) >= vmin && fmaxf(vs0, vs1) < vmax + 1.0f;
        // row v0 = floor(t) as kFloorMagic-biased bits: the pair's address is
        // colb + bits * 8 (colb = col - kFloorBits pairs, 64-bit wrap-around)
        const char* colb = reinterpret_cast<const char*>(col) - size_t(kFloorBits) * sizeof(float2);
        if (inside) {
          const auto fast = [&](int j) {
            const float f = __fadd_rd(fmaf(float(j), dv, vs0), kFloorMagic);
            const float v0 = f - kFloorMagic;
            const float at0 = fabsf(fmaf(v0, Sl, C0) - float(32 * j));
            const float2 yy = __ldg(reinterpret_cast<const float2*>(
                colb + size_t(__float_as_uint(f)) * sizeof(float2)));
            return fmaf(__saturatef(1.0f - at0), yy.x, __saturatef(c1s + at0) * yy.y);
          };
          window_dispatch<kX, kRun, -1>(acc, f0, fast, wl, fa);
        } else {
          // clamping t to [vmin, vmax] (integers; NaN -> vmin) clamps its floor
          const auto clamped = [&](int j) {
            const float t = fminf(fmaxf(fmaf(float(j), dv, vs0), vmin), vmax);
            const float f = __fadd_rd(t, kFloorMagic);
            const float v0 = f - kFloorMagic;
            const float at0 = fabsf(fmaf(v0, Sl, C0) - float(32 * j));
            const float2 yy = __ldg(reinterpret_cast<const float2*>(
                colb + size_t(__float_as_uint(f)) * sizeof(float2)));
            return fmaf(__saturatef(1.0f - at0), yy.x, __saturatef(c1s + at0) * yy.y);
          };
          window_dispatch<kX, kRun, -1>(acc, f0, clamped, wl, fa);
        }
      } else {
        // finer rows than voxels: every row whose tent reaches the voxel
        const auto rows_loop = [&](int j) {
          const float Bj = C0 - float(32 * j);
          const float v1 = (-1.0f - Bj) * inv, v2 = (1.0f - Bj) * inv;
          const int iv_lo = max(0, (int)floorf(clamp_coord(fminf(v1, v2))) + g.ov);
          const int iv_hi = min(g.rows - 1, (int)ceilf(clamp_coord(fmaxf(v1, v2))) + g.ov);
          float acc_v = 0.0f;
          for (int iv = iv_lo; iv <= iv_hi; ++iv)
            acc_v = fmaf(tent(fmaf(float(iv - g.ov), Sl, Bj)), __ldg(col + (iv - g.ov)).x, acc_v);
          return acc_v;
        };
        window_dispatch<kX, kRun, -1>(acc, f0, rows_loop, wl, fa);
      }
    }
  }
  // [y][x][z] scratch: lanes along z, coalesced
#pragma unroll
  for (int m = 0; m < kX; ++m) {
    const int ia = i0 + m;
    if (ia >= n_a) break;
    const size_t base = kAisX ? ((size_t)ip * g.nx + ia) * g.nz : ((size_t)ia * g.nx + ip) * g.nz;
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
      const int z = z0 + 32 * j;
      if (z < g.nz) {
        if (kAdd)
          volt[base + z] = __fadd_rn(volt[base + z], acc[m][j]);
        else
          volt[base + z] = acc[m][j];
      }
    }
  }
}

// Epilogues of the transpose from the [y][x][z] scratch to the caller's volume.
enum ZlaneOut { kOutSet = 0, kOutAdd = 1, kOutSirt = 2 };

// vol[z][y][x] (=, +=) volt[y][x][z], or the SIRT update vol += C * volt with
// the plain recipe's rounding. 32 x 32 tiles of the (x, z) plane of one y
// through shared memory: reads along z and writes along x are both coalesced.
template <int kOut>
__global__ void __launch_bounds__(256)
    bp_zlane_out_kernel(const float* __restrict__ volt, float* __restrict__ vol,
                        const float* __restrict__ C, DeviceGeometry g) {
  __shared__ float tile[32][33];  // [x][z]
  const int z0 = blockIdx.x * 32, x0 = blockIdx.y * 32;
  for (int y = blockIdx.z; y < g.ny; y += gridDim.z) {
    for (int k = threadIdx.y; k < 32; k += 8) {
      const int x = x0 + k, z = z0 + threadIdx.x;
      if (x < g.nx && z < g.nz) tile[k][threadIdx.x] = volt[((size_t)y * g.nx + x) * g.nz + z];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
      const int z = z0 + k, x = x0 + threadIdx.x;
      if (x < g.nx && z < g.nz) {
        const size_t idx = ((size_t)z * g.ny + y) * g.nx + x;
        const float s = tile[threadIdx.x][k];
        if (kOut == kOutSet)
          vol[idx] = s;
        else if (kOut == kOutAdd)
          vol[idx] = __fadd_rn(vol[idx], s);
        else
          vol[idx] = __fadd_rn(vol[idx], __fmul_rn(s, __ldg(C + idx)));
      }
    }
    __syncthreads();
  }
}

template <int kX, int kRun, int kPlanes, int kMinBlocks, bool kAisX>
void launch_zlane_shape(const tsgb_projector* p, const int* angles, int n, bool add,
                        const float2* sinoz, float* volt, cudaStream_t stream) {
  const DeviceGeometry& g = p->g;
  const int n_p = kAisX ? g.ny : g.nx, n_a = kAisX ? g.nx : g.ny;
  const int plane_blocks = (n_p + kPlanes - 1) / kPlanes;
  const long long windows = (n_a + kX - 1) / kX;
  const dim3 grid(unsigned(plane_blocks * windows), unsigned((g.nz + 32 * kRun - 1) / (32 * kRun)));
  if (add)
    bp_zlane_kernel<kX, kRun, kPlanes, kMinBlocks, kAisX, true>
        <<<grid, 32 * kPlanes, 0, stream>>>(p->d_params, p->d_columns, angles, n, sinoz, volt, g,
                                            plane_blocks);
  else
    bp_zlane_kernel<kX, kRun, kPlanes, kMinBlocks, kAisX, false>
        <<<grid, 32 * kPlanes, 0, stream>>>(p->d_params, p->d_columns, angles, n, sinoz, volt, g,
                                            plane_blocks);
}

// Warp shapes chosen by the projector's tuning (window x z run per lane x
// warps per block, minimum resident blocks). Measured on the 512^3 / 1024-angle
// cone scan (ms per backprojection): 4x16x8 124.8, 3x16x8 124.8, 4x16x16 126.1,
// 4x8x4 156, 4x8x8 158, 4x4x4 194, 4x2x4 318 (voxel-pair kernel: 144.5); at
// 256^3 / 360 angles 4x8x4 and 4x8x8 7.2 (voxel-pair kernel 6.76), the 16-z
// shapes about 13 (half of each warp's 512 z lie outside the volume).
template <bool kAisX>
void launch_zlane_pass(const tsgb_projector* p, const int* angles, int n, bool add,
                       const float2* sinoz, float* volt, cudaStream_t stream) {
  switch (zlane_shape(p)) {
    case 1:
      launch_zlane_shape<4, 8, 8, 3, kAisX>(p, angles, n, add, sinoz, volt, stream);
      break;
    case 2:
      launch_zlane_shape<4, 16, 8, 2, kAisX>(p, angles, n, add, sinoz, volt, stream);
      break;
    case 3:
      launch_zlane_shape<4, 16, 16, 1, kAisX>(p, angles, n, add, sinoz, volt, stream);
      break;
    case 4:
      launch_zlane_shape<3, 16, 8, 2, kAisX>(p, angles, n, add, sinoz, volt, stream);
      break;
    case 5:
      launch_zlane_shape<4, 4, 4, 6, kAisX>(p, angles, n, add, sinoz, volt, stream);
      break;
    case 6:
      launch_zlane_shape<4, 2, 4, 6, kAisX>(p, angles, n, add, sinoz, volt, stream);
      break;
    default:
      launch_zlane_shape<4, 8, 4, 6, kAisX>(p, angles, n, add, sinoz, volt, stream);
  }
}

void launch_zlane_out(const tsgb_projector* p, int mode, const float* volt, float* vol,
                      const float* C, cudaStream_t stream) {
  const DeviceGeometry& g = p->g;
  const dim3 grid(unsigned((g.nz + 31) / 32), unsigned((g.nx + 31) / 32),
                  unsigned(std::min(g.ny, 65535)));
  const dim3 block(32, 8);
  if (mode == kOutSet)
    bp_zlane_out_kernel<kOutSet><<<grid, block, 0, stream>>>(volt, vol, C, g);
  else if (mode == kOutAdd)
    bp_zlane_out_kernel<kOutAdd><<<grid, block, 0, stream>>>(volt, vol, C, g);
  else
    bp_zlane_out_kernel<kOutSirt><<<grid, block, 0, stream>>>(volt, vol, C, g);
}

}  // namespace

int64_t bp_pairs_bytes(const DeviceGeometry& g) {
  return (int64_t(g.rows + 2 * kRowPad) * g.nangles * g.cols * 8 + 255) / 256 * 256;
}

int64_t bp_volume_bytes(const DeviceGeometry& g) {
  return (int64_t(g.nz) * g.ny * g.nx * 4 + 255) / 256 * 256;
}

int launch_bp_weight_z(const tsgb_projector* p, const float* sino, float* sinoz_f,
                       int angle_begin, int angle_end, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  float2* sinoz = reinterpret_cast<float2*>(sinoz_f);
  const DeviceGeometry& g = p->g;
  const int RP = g.rows + 2 * kRowPad;
  for (int a0 = angle_begin; a0 < angle_end; a0 += 65535) {
    const int n = std::min(angle_end - a0, 65535);
    const dim3 grid(unsigned((g.cols + 31) / 32), unsigned((RP + 31) / 32), unsigned(n));
    bp_weight_z_kernel<<<grid, dim3(32, 8), 0, stream>>>(
        p->d_params, p->d_columns, sino, sinoz + (size_t)a0 * g.cols * RP, g, a0);
  }
  return int(cudaGetLastError());
}

bool launch_bp_zlane_separable(const tsgb_projector* p, int off_x, int n_ax, int off_y, int n_ay,
                               const float* sinoz_f, float* volt, float* vol, int out_mode,
                               const float* C, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const float2* sinoz = reinterpret_cast<const float2*>(sinoz_f);
  if (n_ax + n_ay == 0) return false;
  // both passes into volt, the second adding onto the first
  if (n_ax > 0) launch_zlane_pass<true>(p, p->d_sep_angles + off_x, n_ax, false, sinoz, volt, stream);
  if (n_ay > 0)
    launch_zlane_pass<false>(p, p->d_sep_angles + off_y, n_ay, n_ax > 0, sinoz, volt, stream);
  launch_zlane_out(p, out_mode, volt, vol, C, stream);
  return true;
}

}  // namespace tsgb
