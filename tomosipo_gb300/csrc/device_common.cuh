// Device helpers shared by the projector kernels.
#pragma once

#include <cuda_runtime.h>

#include "tsgb_internal.h"

namespace tsgb {

// Per-layout description of a padded forward-projection volume copy, laid
// out [d][a][b] (b fastest) with kPad zero voxels on both sides of a and b.
struct LayoutDev {
  long long offset;
  int n_d, n_a, n_b;
  int o_d, o_a, o_b;
  int stride_d, stride_a;
};

struct LayoutTable {
  LayoutDev l[kMaxLayouts];
  int count;
};

__host__ inline LayoutTable make_layout_table(const tsgb_projector* p) {
  LayoutTable t{};
  const int anchors[3] = {p->g.oz, p->g.oy, p->g.ox};
  t.count = int(p->layouts.size());
  for (int i = 0; i < t.count; ++i) {
    const Layout& L = p->layouts[i];
    LayoutDev& D = t.l[i];
    D.offset = L.offset_elems;
    D.n_d = int(L.n_d);
    D.n_a = int(L.n_a);
    D.n_b = int(L.n_b);
    D.o_d = anchors[L.d];
    D.o_a = anchors[L.a];
    D.o_b = anchors[L.b];
    D.stride_a = int(L.n_b + 2 * kPad);
    D.stride_d = int((L.n_a + 2 * kPad) * (L.n_b + 2 * kPad));
  }
  return t;
}

// Ray through anchored pixel (ut, vt) for one angle: in-plane position on
// plane kt of the dominant axis is (Xa + kt ma, Xb + kt mb).
struct Ray {
  float Xa, ma, Xb, mb;
};

__device__ __forceinline__ Ray ray_general(const AngleParams& ap, float ut, float vt) {
  const float den = fmaf(ap.e[2], vt, fmaf(ap.e[1], ut, ap.e[0]));
  const float inv = 1.0f / den;
  Ray r;
  r.Xa = fmaf(ap.ca[2], vt, fmaf(ap.ca[1], ut, ap.ca[0])) * inv;
  r.ma = fmaf(ap.ma[2], vt, fmaf(ap.ma[1], ut, ap.ma[0])) * inv;
  r.Xb = fmaf(ap.cb[2], vt, fmaf(ap.cb[1], ut, ap.cb[0])) * inv;
  r.mb = fmaf(ap.mb[2], vt, fmaf(ap.mb[1], ut, ap.mb[0])) * inv;
  return r;
}

__device__ __forceinline__ Ray ray_column(const ColumnEntry& c, float vt) {
  Ray r;
  r.Xa = c.Xa;
  r.ma = c.ma;
  r.Xb = fmaf(vt, c.R, c.P);
  r.mb = fmaf(vt, c.S, c.Q);
  return r;
}

// World length of the ray between consecutive planes of the dominant axis.
__device__ __forceinline__ float ray_step(const AngleParams& ap, const Ray& r) {
  const float vd = ap.vs_d, va = ap.vs_a * r.ma, vb = ap.vs_b * r.mb;
  return sqrtf(fmaf(vd, vd, fmaf(va, va, vb * vb)));
}

// Job of block b in a multi-job launch: the j with start[j] <= b < start[j + 1]
// (start[0] = 0, n jobs).
__device__ __forceinline__ int multi_job_of(const long long* start, int n, long long b) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (b >= start[mid])
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ float tent(float t) { return fmaxf(0.0f, 1.0f - fabsf(t)); }

// Exact floor without the conversion unit: for |t| < 2^22, t + 1.5 * 2^23
// rounded toward -inf (__fadd_rd) is floor(t) + 1.5 * 2^23, an integer-valued
// float (floats there are spaced by 1) whose bit pattern is 0x4B400000 +
// floor(t). So floor(t) as a float is that sum minus kFloorMagic, and as an
// integer its bits minus kFloorBits: add and integer instructions, where
// floorf plus a float-to-int conversion would occupy the conversion (XU) pipe.
constexpr float kFloorMagic = 12582912.0f;
constexpr unsigned kFloorBits = 0x4B400000u;

// Clamp a detector coordinate to +-1e8 before an int conversion (NaN -> -1e8,
// +-inf -> +-1e8), so range bounds never overflow 32-bit integers.
__device__ __forceinline__ float clamp_coord(float c) { return fminf(fmaxf(c, -1.0e8f), 1.0e8f); }

__device__ __forceinline__ bool finite_ray(const Ray& r) {
  return isfinite(r.Xa) && isfinite(r.ma) && isfinite(r.Xb) && isfinite(r.mb);
}

// ------------------------------------------------------------ FP tile order
// Tile (row block, column block, angle pair) of linear block b under s. The
// blocks of a group of pairs come first, inside a group the patches strip by
// strip, inside a patch the pairs and then the tiles with row blocks fastest.
// Only the last group, strip and patch can be smaller than the others, so
// each level's index is a plain quotient.
__device__ __forceinline__ void fp_schedule_tile(const FpSchedule& s, long long b, int& rb,
                                                 int& cb, int& pair) {
  const long long per_pair = (long long)s.row_blocks * s.col_blocks;
  const long long full_group = per_pair * s.group_pairs;
  const int grp = int(b / full_group);
  b -= grp * full_group;
  const int gsz = min(s.group_pairs, s.pairs - grp * s.group_pairs);
  const long long full_strip = (long long)gsz * s.patch_rows * s.col_blocks;
  const int pr = int(b / full_strip);
  b -= pr * full_strip;
  const int rsz = min(s.patch_rows, s.row_blocks - pr * s.patch_rows);
  const long long full_patch = (long long)gsz * rsz * s.patch_cols;
  const int pc = int(b / full_patch);
  b -= pc * full_patch;
  const int csz = min(s.patch_cols, s.col_blocks - pc * s.patch_cols);
  const long long tiles = (long long)rsz * csz;
  const long long q = b / tiles;
  pair = grp * s.group_pairs + int(q);
  const int t = int(b - q * tiles);
  rb = pr * s.patch_rows + t % rsz;
  cb = pc * s.patch_cols + t / rsz;
}

}  // namespace tsgb
