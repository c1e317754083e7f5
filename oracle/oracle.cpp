// FP64 CPU oracle of the tomosipo_gb300 projector -- TEST INFRASTRUCTURE ONLY.
//
// Only the tests, the smoke check and the CPU-baseline leg of bench.py use
// this file, as the reference the results are compared with and as the timed
// CPU baseline. The product path never calls it.
//
// What it restates. tomosipo delegates A(x) / A.T(y) to ASTRA's cuda3d
// projector (tomosipo/astra.py:80-98, 147-153); ASTRA is a third-party
// dependency ("astra-toolbox>=2.0", setup.py:14-17, not pinned, not vendored,
// not installed here), so this oracle restates the discretisation the
// GB300 kernels implement, written independently of them:
//  * geometry conventions of tomosipo: volume voxel centres at
//    pos - size/2 + (i + 1/2) size/shape (tomosipo/geometry/volume_vec.py:386-399);
//    pixel centres at det_pos + (iv + 1/2 - rows/2) det_v + (iu + 1/2 - cols/2) det_u
//    (tomosipo/geometry/det_vec.py:301-322); sinogram layout (rows, angles, cols)
//    (tomosipo/links/base.py:21-31).
//  * forward projection (Joseph's method): per angle a dominant axis d, the
//    largest component of the central ray in voxel units; every ray is sampled
//    on each voxel-centre plane of d, bilinearly in the other two axes with
//    zeros outside the volume, and the sum is scaled by the world length of
//    one plane step. Rays steeper than 64 voxels per plane are not sampled.
//  * matched backprojection: the literal transpose, computed by scattering
//    every ray's weights back onto the volume.
//  * bilinear backprojection: voxel-driven; the detector is interpolated
//    bilinearly at the projection of each (sub-)voxel centre and weighted by
//    voxel volume / pixel area / |cos| of the ray to the detector normal
//    (times the squared cone magnification).
// Everything is computed in double precision from the world-space vectors.
//
// Parity pin. No golden FP/BP vectors exist in the reference (its tests are
// relational, tests/test_Operator.py, tests/test_torch_support.py), so the
// oracle is pinned by the reference's one numeric FP output (the hollow-box
// sinogram mean and maximum in notebooks/cupy.ipynb, cell 4), by analytic
// known answers (chord lengths), by exact identities (adjointness, mirrored
// opposite angles, quarter-turns, whole-voxel shifts, scaling) and by the
// reference's own geometry conventions; see tests/test_oracle.py.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "tomosipo_gb300.h"

namespace {

struct Geo {
  int64_t n[3];
  double vs[3], llc[3];
  int kind, rows, cols;
  int64_t nangles;
  const double* vec;
};

Geo make_geo(const tsgb_volume_desc* v, const tsgb_projection_desc* p) {
  Geo g;
  for (int i = 0; i < 3; ++i) {
    g.n[i] = v->shape[i];
    g.vs[i] = v->size[i] / double(v->shape[i]);
    g.llc[i] = v->pos[i] - 0.5 * v->size[i];
  }
  g.kind = p->kind;
  g.rows = int(p->det_shape[0]);
  g.cols = int(p->det_shape[1]);
  g.nangles = p->num_angles;
  g.vec = p->vectors;
  return g;
}

// world point -> voxel index coordinates (voxel i centred at i)
void to_index(const Geo& g, const double* w, double* out) {
  for (int i = 0; i < 3; ++i) out[i] = (w[i] - g.llc[i]) / g.vs[i] - 0.5;
}

int dominant_axis(const Geo& g, const double* row) {
  double ref[3];
  for (int i = 0; i < 3; ++i)
    ref[i] = (g.kind == TSGB_CONE ? row[3 + i] - row[i] : row[i]) / g.vs[i];
  int d = 0;
  for (int i = 1; i < 3; ++i)
    if (std::fabs(ref[i]) > std::fabs(ref[d])) d = i;
  return d;
}

// Visit every (voxel, weight) pair of one ray: origin o and direction r in
// voxel index coordinates, dominant axis d. Only voxels with z in
// [z_lo, z_hi) are visited (the full range by default). f(flat_index, weight).
template <typename F>
void walk_ray(const Geo& g, int d, const double* o, const double* r, F&& f, int64_t z_lo = 0,
              int64_t z_hi = -1) {
  if (z_hi < 0) z_hi = g.n[0];
  const int a = d == 0 ? 1 : 0;  // for d != 0 the first in-plane axis is z
  const int b = d == 2 ? 1 : 2;
  if (r[d] == 0.0) return;
  const double sa = r[a] / r[d], sb = r[b] / r[d];
  if (!(std::fabs(sa) <= 64.0) || !(std::fabs(sb) <= 64.0)) return;
  double step2 = 0.0;
  for (int i = 0; i < 3; ++i) {
    const double c = g.vs[i] * r[i] / r[d];
    step2 += c * c;
  }
  const double step = std::sqrt(step2);
  const int64_t stride[3] = {g.n[1] * g.n[2], g.n[2], 1};
  // planes whose z taps can reach [z_lo, z_hi)
  int64_t k0 = 0, k1 = g.n[d] - 1;
  if (d == 0) {
    k0 = std::max<int64_t>(k0, z_lo);
    k1 = std::min<int64_t>(k1, z_hi - 1);
  } else if (z_lo > 0 || z_hi < g.n[0]) {
    // z(k) = o[0] + (k - o[d]) * sa must lie in (z_lo - 1, z_hi)
    if (sa == 0.0) {
      if (!(o[0] > z_lo - 1 && o[0] < z_hi)) return;
    } else {
      double t1 = o[d] + (z_lo - 1 - o[0]) / sa, t2 = o[d] + (z_hi - o[0]) / sa;
      if (t1 > t2) std::swap(t1, t2);
      k0 = std::max<int64_t>(k0, int64_t(std::floor(std::max(t1, -1.0))));
      k1 = std::min<int64_t>(k1, int64_t(std::ceil(std::min(t2, double(g.n[d])))));
    }
  }
  for (int64_t k = k0; k <= k1; ++k) {
    const double t = (double(k) - o[d]) / r[d];
    const double qa = o[a] + t * r[a], qb = o[b] + t * r[b];
    const double fa = std::floor(qa), fb = std::floor(qb);
    const int64_t ia = int64_t(fa), ib = int64_t(fb);
    const double wa1 = qa - fa, wb1 = qb - fb;
    for (int da = 0; da < 2; ++da) {
      const int64_t i = ia + da;
      if (i < 0 || i >= g.n[a]) continue;
      if (d != 0 && (i < z_lo || i >= z_hi)) continue;  // a == z here
      const double wa = da ? wa1 : 1.0 - wa1;
      for (int db = 0; db < 2; ++db) {
        const int64_t j = ib + db;
        if (j < 0 || j >= g.n[b]) continue;
        const double wb = db ? wb1 : 1.0 - wb1;
        const double w = wa * wb * step;
        if (w != 0.0) f(k * stride[d] + i * stride[a] + j * stride[b], w);
      }
    }
  }
}

// Ray of sub-pixel (s_v, s_u) of pixel (iv, iu) at angle t.
void make_ray(const Geo& g, int64_t t, int iv, int iu, double sv, double su, double* o,
              double* r) {
  const double* row = g.vec + 12 * t;
  double p[3];
  for (int i = 0; i < 3; ++i)
    p[i] = row[3 + i] + (iv + 0.5 + sv - 0.5 * g.rows) * row[6 + i] +
           (iu + 0.5 + su - 0.5 * g.cols) * row[9 + i];
  to_index(g, p, o);
  if (g.kind == TSGB_CONE) {
    double s[3];
    to_index(g, row, s);
    for (int i = 0; i < 3; ++i) r[i] = o[i] - s[i];
  } else {
    for (int i = 0; i < 3; ++i) r[i] = row[i] / g.vs[i];
  }
}

template <typename F>
void parallel_for(int64_t n, int nthreads, F&& f) {
  nthreads = std::max(1, nthreads);
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t)
    pool.emplace_back([&, t] {
      for (int64_t i = t; i < n; i += nthreads) f(i, t);
    });
  for (auto& th : pool) th.join();
}

int check(const tsgb_volume_desc* v, const tsgb_projection_desc* p) {
  if (!v || !p || !p->vectors) return -1;
  if (p->kind != TSGB_CONE && p->kind != TSGB_PARALLEL) return -1;
  for (int i = 0; i < 3; ++i)
    if (v->shape[i] < 1 || !(v->size[i] > 0)) return -1;
  if (p->det_shape[0] < 1 || p->det_shape[1] < 1 || p->num_angles < 1) return -1;
  return 0;
}

}  // namespace

extern "C" {

// sino[rows][angles][cols] = A vol, with det_ss x det_ss rays per pixel averaged.
// Parallel over (angle, detector row).
int oracle_fp(const tsgb_volume_desc* v, const tsgb_projection_desc* p, int det_ss,
              const double* vol, double* sino, int nthreads) {
  if (check(v, p) || det_ss < 1) return -1;
  const Geo g = make_geo(v, p);
  const double inv = 1.0 / (double(det_ss) * det_ss);
  parallel_for(g.nangles * g.rows, nthreads, [&](int64_t item, int) {
    const int64_t t = item / g.rows;
    const int iv = int(item % g.rows);
    const int d = dominant_axis(g, g.vec + 12 * t);
    for (int iu = 0; iu < g.cols; ++iu) {
      double acc = 0.0;
      for (int s1 = 0; s1 < det_ss; ++s1)
        for (int s2 = 0; s2 < det_ss; ++s2) {
          double o[3], r[3];
          make_ray(g, t, iv, iu, (s1 + 0.5) / det_ss - 0.5, (s2 + 0.5) / det_ss - 0.5, o, r);
          walk_ray(g, d, o, r, [&](int64_t idx, double w) { acc += w * vol[idx]; });
        }
      sino[(int64_t(iv) * g.nangles + t) * g.cols + iu] = acc * inv;
    }
  });
  return 0;
}

// vol = A^T sino: the exact transpose of oracle_fp, by scattering every ray's
// weights. Parallel over disjoint z slabs: each thread walks every ray but
// only visits the voxels of its own slab, so no two threads write the same
// voxel and the summation order is fixed (deterministic).
int oracle_bp_matched(const tsgb_volume_desc* v, const tsgb_projection_desc* p, int det_ss,
                      const double* sino, double* vol, int nthreads) {
  if (check(v, p) || det_ss < 1) return -1;
  const Geo g = make_geo(v, p);
  const int64_t nvox = g.n[0] * g.n[1] * g.n[2];
  std::fill(vol, vol + nvox, 0.0);
  const double inv = 1.0 / (double(det_ss) * det_ss);
  const int64_t nslab = std::min<int64_t>(g.n[0], std::max(1, nthreads) * 2);
  parallel_for(nslab, nthreads, [&](int64_t slab, int) {
    const int64_t z_lo = g.n[0] * slab / nslab, z_hi = g.n[0] * (slab + 1) / nslab;
    for (int64_t t = 0; t < g.nangles; ++t) {
      const int d = dominant_axis(g, g.vec + 12 * t);
      for (int iv = 0; iv < g.rows; ++iv)
        for (int iu = 0; iu < g.cols; ++iu) {
          const double y = sino[(int64_t(iv) * g.nangles + t) * g.cols + iu] * inv;
          if (y == 0.0) continue;
          for (int s1 = 0; s1 < det_ss; ++s1)
            for (int s2 = 0; s2 < det_ss; ++s2) {
              double o[3], r[3];
              make_ray(g, t, iv, iu, (s1 + 0.5) / det_ss - 0.5, (s2 + 0.5) / det_ss - 0.5, o, r);
              walk_ray(g, d, o, r, [&](int64_t idx, double w) { vol[idx] += w * y; }, z_lo, z_hi);
            }
        }
    }
  });
  return 0;
}

// vol = voxel-driven bilinear backprojection with vox_ss^3 points per voxel.
int oracle_bp_bilinear(const tsgb_volume_desc* v, const tsgb_projection_desc* p, int vox_ss,
                       const double* sino, double* vol, int nthreads) {
  if (check(v, p) || vox_ss < 1) return -1;
  const Geo g = make_geo(v, p);
  const double vvox = g.vs[0] * g.vs[1] * g.vs[2];
  parallel_for(g.n[0], nthreads, [&](int64_t iz, int) {
    for (int64_t iy = 0; iy < g.n[1]; ++iy)
      for (int64_t ix = 0; ix < g.n[2]; ++ix) {
        double acc = 0.0;
        for (int64_t t = 0; t < g.nangles; ++t) {
          const double* row = g.vec + 12 * t;
          const double* src = row;
          const double* det = row + 3;
          const double* dv = row + 6;
          const double* du = row + 9;
          // normal n = du x dv (same component order as the kernels' host code)
          const double n[3] = {du[1] * dv[2] - du[2] * dv[1], du[2] * dv[0] - du[0] * dv[2],
                               du[0] * dv[1] - du[1] * dv[0]};
          const double area = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
          for (int sz = 0; sz < vox_ss; ++sz)
            for (int sy = 0; sy < vox_ss; ++sy)
              for (int sx = 0; sx < vox_ss; ++sx) {
                const double off[3] = {(sz + 0.5) / vox_ss, (sy + 0.5) / vox_ss,
                                       (sx + 0.5) / vox_ss};
                const int64_t idx[3] = {iz, iy, ix};
                double P[3];
                for (int i = 0; i < 3; ++i) P[i] = g.llc[i] + (idx[i] + off[i]) * g.vs[i];
                double dir[3];
                for (int i = 0; i < 3; ++i) dir[i] = g.kind == TSGB_CONE ? P[i] - src[i] : src[i];
                const double dn = dir[0] * n[0] + dir[1] * n[1] + dir[2] * n[2];
                if (dn == 0.0) continue;
                // hit = P + t dir on the detector plane
                const double tt = ((det[0] - P[0]) * n[0] + (det[1] - P[1]) * n[1] +
                                   (det[2] - P[2]) * n[2]) / dn;
                double hit[3];
                for (int i = 0; i < 3; ++i) hit[i] = P[i] + tt * dir[i] - det[i];
                // solve hit = a du + b dv (least squares on the 2x2 Gram system)
                const double uu = du[0] * du[0] + du[1] * du[1] + du[2] * du[2];
                const double vv = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
                const double uv = du[0] * dv[0] + du[1] * dv[1] + du[2] * dv[2];
                const double hu = hit[0] * du[0] + hit[1] * du[1] + hit[2] * du[2];
                const double hv = hit[0] * dv[0] + hit[1] * dv[1] + hit[2] * dv[2];
                const double det2 = uu * vv - uv * uv;
                const double cu = (hu * vv - hv * uv) / det2;
                const double cv = (hv * uu - hu * uv) / det2;
                // continuous pixel index (centre of pixel i at i)
                const double fu = cu + 0.5 * g.cols - 0.5, fv = cv + 0.5 * g.rows - 0.5;
                const double u0 = std::floor(fu), v0 = std::floor(fv);
                const double wu = fu - u0, wv = fv - v0;
                double val = 0.0;
                for (int a = 0; a < 2; ++a)
                  for (int b = 0; b < 2; ++b) {
                    const int64_t ju = int64_t(u0) + a, jv = int64_t(v0) + b;
                    if (ju < 0 || ju >= g.cols || jv < 0 || jv >= g.rows) continue;
                    val += (a ? wu : 1 - wu) * (b ? wv : 1 - wv) *
                           sino[(jv * g.nangles + t) * g.cols + ju];
                  }
                const double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
                const double cosphi = std::fabs(dn) / (len * area);
                double c = vvox / (area * cosphi);
                if (g.kind == TSGB_CONE) {
                  const double mag = 1.0 + tt;  // (hit - src) / (P - src) along the ray
                  if (mag <= 0.0) continue;     // detector plane behind the source
                  c *= mag * mag;
                }
                acc += c * val;
              }
        }
        vol[(iz * g.n[1] + iy) * g.n[2] + ix] = acc / (double(vox_ss) * vox_ss * vox_ss);
      }
  });
  return 0;
}

}  // extern "C"
