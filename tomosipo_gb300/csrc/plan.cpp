// Host-side (fp64) construction of the per-angle projector tables.
//
// Input is what tomosipo hands ASTRA in ``create_astra_projector``
// (tomosipo/astra.py:80-98): an axis-aligned volume and the vector form of
// the projection geometry. Everything here runs once per projector, in
// double precision, and is rounded to fp32 only at the end so the kernels
// start from correctly rounded coefficients.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "tsgb_internal.h"

namespace tsgb {
namespace {

struct V3 {
  double c[3];
  double& operator[](int i) { return c[i]; }
  double operator[](int i) const { return c[i]; }
};

V3 sub(const V3& a, const V3& b) { return {{a[0] - b[0], a[1] - b[1], a[2] - b[2]}}; }
double dot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
// Cross product on the stored components; only used inside ratios of triple
// products, which do not depend on the handedness of the component order.
V3 cross(const V3& a, const V3& b) {
  return {{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]}};
}
double norm(const V3& a) { return std::sqrt(dot(a, a)); }
V3 scale(const V3& a, double s) { return {{a[0] * s, a[1] * s, a[2] * s}}; }
V3 axpy(const V3& a, double s, const V3& b) {  // a + s * b
  return {{a[0] + s * b[0], a[1] + s * b[1], a[2] + s * b[2]}};
}

int argmax_abs(const V3& v, int skip) {
  int best = -1;
  for (int i = 0; i < 3; ++i) {
    if (i == skip) continue;
    if (best < 0 || std::fabs(v[i]) > std::fabs(v[best])) best = i;
  }
  return best;
}

bool finite3(const V3& v) {
  return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

}  // namespace

std::string reduce_angle(const double* row, bool cone, const double vs[3], const double origin[3],
                         int rows, int cols, int ov, int ou, bool allow_separable, int t,
                         AngleFrame* f) {
  V3 src_w{{row[0], row[1], row[2]}}, det_w{{row[3], row[4], row[5]}};
  V3 v_w{{row[6], row[7], row[8]}}, u_w{{row[9], row[10], row[11]}};
  if (!finite3(src_w) || !finite3(det_w) || !finite3(v_w) || !finite3(u_w))
    return "non-finite geometry vector at angle " + std::to_string(t);
  if (norm(u_w) == 0.0 || norm(v_w) == 0.0 || norm(cross(u_w, v_w)) == 0.0)
    return "degenerate detector pixel vectors at angle " + std::to_string(t);
  // Anchored pixel origin: centre of pixel (ov, ou) (world units).
  const V3 dc_w = axpy(axpy(det_w, ov + 0.5 - 0.5 * rows, v_w), ou + 0.5 - 0.5 * cols, u_w);
  V3 ref;  // central ray direction in voxel units
  for (int i = 0; i < 3; ++i) {
    f->U[i] = u_w[i] / vs[i];
    f->V[i] = v_w[i] / vs[i];
    f->Dc[i] = (dc_w[i] - origin[i]) / vs[i];
    f->S[i] = (src_w[i] - origin[i]) / vs[i];  // source (cone)
    f->R[i] = src_w[i] / vs[i];                // ray direction (parallel)
    ref[i] = cone ? (det_w[i] - src_w[i]) / vs[i] : f->R[i];
  }
  if (norm(ref) == 0.0) return "zero ray direction at angle " + std::to_string(t);
  const int d = argmax_abs(ref, -1);
  const V3 Vv{{f->V[0], f->V[1], f->V[2]}};
  const int b = argmax_abs(Vv, d);
  const int a = 3 - d - b;
  f->d = d;
  f->a = a;
  f->b = b;
  const double vn = norm(Vv);
  f->separable = allow_separable && std::fabs(f->V[d]) <= 1e-12 * vn &&
                 std::fabs(f->V[a]) <= 1e-12 * vn;
  if (f->separable) {
    f->V[d] = 0.0;
    f->V[a] = 0.0;
  }
  // Ray coefficients over (1, ut, vt).
  if (cone) {
    const double D[3] = {f->Dc[0] - f->S[0], f->Dc[1] - f->S[1], f->Dc[2] - f->S[2]};
    if (D[d] == 0.0) return "detector centre lies in the source's dominant plane";
    const double sc = 1.0 / D[d];  // normalise so den = 1 at the anchored pixel
    const double ed[3] = {D[d], f->U[d], f->V[d]};
    const double ea[3] = {D[a], f->U[a], f->V[a]};
    const double eb[3] = {D[b], f->U[b], f->V[b]};
    for (int j = 0; j < 3; ++j) {
      f->e[j] = ed[j] * sc;
      f->ca[j] = (f->S[a] * ed[j] - f->S[d] * ea[j]) * sc;
      f->ma[j] = ea[j] * sc;
      f->cb[j] = (f->S[b] * ed[j] - f->S[d] * eb[j]) * sc;
      f->mb[j] = eb[j] * sc;
    }
  } else {
    if (f->R[d] == 0.0) return "ray parallel to every volume plane";
    const double sa = f->R[a] / f->R[d], sb = f->R[b] / f->R[d];
    f->e[0] = 1.0;
    f->e[1] = f->e[2] = 0.0;
    f->ca[0] = f->Dc[a] - f->Dc[d] * sa;
    f->ca[1] = f->U[a] - f->U[d] * sa;
    f->ca[2] = f->V[a] - f->V[d] * sa;
    f->cb[0] = f->Dc[b] - f->Dc[d] * sb;
    f->cb[1] = f->U[b] - f->U[d] * sb;
    f->cb[2] = f->V[b] - f->V[d] * sb;
    f->ma[0] = sa;
    f->mb[0] = sb;
    f->ma[1] = f->ma[2] = f->mb[1] = f->mb[2] = 0.0;
  }
  return std::string();
}

std::string build_plan(const tsgb_volume_desc* vol, const tsgb_projection_desc* proj,
                       int voxel_ss, int det_ss, tsgb_projector* p,
                       std::vector<ColumnEntry>* columns, std::vector<int>* sep_angles,
                       std::vector<int>* gen_angles, std::vector<int>* bil_fast,
                       std::vector<int>* bil_slow) {
  if (!vol || !proj || !proj->vectors) return "null geometry descriptor";
  if (proj->kind != TSGB_PARALLEL && proj->kind != TSGB_CONE)
    return "projection kind must be TSGB_PARALLEL or TSGB_CONE";
  if (voxel_ss < 1 || det_ss < 1 || voxel_ss > 16 || det_ss > 16)
    return "supersampling factors must lie in [1, 16]";
  if (det_ss != 1) return "the plan is built per detector; supersampling is a finer detector";
  for (int i = 0; i < 3; ++i) {
    if (vol->shape[i] < 1 || vol->shape[i] > (1 << 20)) return "volume shape out of range";
    if (!(vol->size[i] > 0) || !std::isfinite(vol->size[i]) || !std::isfinite(vol->pos[i]))
      return "volume size must be positive and finite";
  }
  if (proj->det_shape[0] < 1 || proj->det_shape[1] < 1 || proj->det_shape[0] > (1 << 20) ||
      proj->det_shape[1] > (1 << 20))
    return "detector shape out of range";
  if (proj->num_angles < 1 || proj->num_angles > (1 << 24)) return "number of angles out of range";
  const int64_t nvox = vol->shape[0] * vol->shape[1] * vol->shape[2];
  const int64_t nsino = proj->det_shape[0] * proj->det_shape[1] * proj->num_angles;
  if (nvox > (int64_t(1) << 40) || nsino > (int64_t(1) << 40)) return "data too large";

  DeviceGeometry& g = p->g;
  g.kind = proj->kind;
  g.nz = int(vol->shape[0]);
  g.ny = int(vol->shape[1]);
  g.nx = int(vol->shape[2]);
  g.oz = g.nz / 2;
  g.oy = g.ny / 2;
  g.ox = g.nx / 2;
  g.rows = int(proj->det_shape[0]);
  g.cols = int(proj->det_shape[1]);
  g.nangles = int(proj->num_angles);
  g.ov = g.rows / 2;
  g.ou = g.cols / 2;
  g.det_ss = det_ss;
  g.vox_ss = voxel_ss;
  const int shape[3] = {g.nz, g.ny, g.nx};
  const int anchor[3] = {g.oz, g.oy, g.ox};
  V3 vs, origin;
  for (int i = 0; i < 3; ++i) {
    vs[i] = vol->size[i] / double(vol->shape[i]);
    g.vs[i] = float(vs[i]);
    // world position of the anchor voxel's centre
    origin[i] = vol->pos[i] - 0.5 * vol->size[i] + (anchor[i] + 0.5) * vs[i];
  }
  const double vox_volume = vs[0] * vs[1] * vs[2];
  const bool cone = proj->kind == TSGB_CONE;

  p->host_params.assign(g.nangles, AngleParams{});
  p->layouts.clear();
  columns->assign(size_t(g.nangles) * g.cols, ColumnEntry{});
  sep_angles->clear();
  p->fine_rows = false;
  double fine_planes = 0.0, all_planes = 0.0;  // (separable angle, column, plane) triples
  gen_angles->clear();
  bil_fast->clear();
  bil_slow->clear();

  const double vs_a[3] = {vs[0], vs[1], vs[2]}, origin_a[3] = {origin[0], origin[1], origin[2]};
  for (int t = 0; t < g.nangles; ++t) {
    const double* row = proj->vectors + 12 * size_t(t);
    AngleFrame f;
    const std::string err =
        reduce_angle(row, cone, vs_a, origin_a, g.rows, g.cols, g.ov, g.ou, det_ss == 1, t, &f);
    if (!err.empty()) return err;
    const V3 u_w{{row[9], row[10], row[11]}}, v_w{{row[6], row[7], row[8]}};
    const V3 src_w{{row[0], row[1], row[2]}};
    const V3 U{{f.U[0], f.U[1], f.U[2]}}, V{{f.V[0], f.V[1], f.V[2]}};
    const V3 Dc{{f.Dc[0], f.Dc[1], f.Dc[2]}}, S{{f.S[0], f.S[1], f.S[2]}};
    const V3 R{{f.R[0], f.R[1], f.R[2]}};
    AngleParams& ap = p->host_params[t];
    const int d = f.d, a = f.a, b = f.b;
    ap.d = d;
    ap.a = a;
    ap.b = b;
    const bool separable = f.separable;
    ap.separable = separable ? 1 : 0;
    const double *e = f.e, *ca = f.ca, *ma = f.ma, *cb = f.cb, *mb = f.mb;
    for (int j = 0; j < 3; ++j) {
      ap.e[j] = float(e[j]);
      ap.ca[j] = float(ca[j]);
      ap.ma[j] = float(ma[j]);
      ap.cb[j] = float(cb[j]);
      ap.mb[j] = float(mb[j]);
    }

    // Voxel -> detector projection, anchored coordinates in (z, y, x) order.
    double pu[4], pv[4], pw[4];
    if (cone) {
      V3 r = sub(Dc, S);
      V3 nu = cross(V, r), nv = cross(r, U), nw = cross(U, V);
      const double den0 = -dot(S, nw);
      if (den0 == 0.0) return "source lies in the detector plane's parallel through the volume";
      for (int i = 0; i < 3; ++i) {
        pu[i] = nu[i] / den0;
        pv[i] = nv[i] / den0;
        pw[i] = nw[i] / den0;
      }
      pu[3] = -dot(S, nu) / den0;
      pv[3] = -dot(S, nv) / den0;
      pw[3] = 1.0;
      // Bilinear weight: K^2 / |den0|^3 * |P - S|_world / dn^3 (see header).
      const double K = dot(r, nw);
      ap.bil_scale = float(K * K / std::fabs(den0 * den0 * den0));
    } else {
      V3 rv = cross(R, V), ur = cross(U, R);
      const double den = dot(R, cross(U, V));
      if (den == 0.0) return "ray direction lies in the detector plane";
      for (int i = 0; i < 3; ++i) {
        pu[i] = -rv[i] / den;
        pv[i] = -ur[i] / den;
        pw[i] = 0.0;
      }
      pu[3] = dot(Dc, rv) / den;
      pv[3] = dot(Dc, ur) / den;
      pw[3] = 1.0;
      V3 nw_w = cross(u_w, v_w);
      ap.bil_scale = float(vox_volume * norm(src_w) / std::fabs(dot(src_w, nw_w)));
    }
    for (int i = 0; i < 4; ++i) {
      ap.pu[i] = float(pu[i]);
      ap.pv[i] = float(pv[i]);
      ap.pw[i] = float(pw[i]);
    }
    // Exact zeros when det_v runs along z (V = (v, 0, 0)): then u and the
    // projective denominator are constant along a voxel column in z.
    // the z-flat kernel's quad copy needs 32-bit offsets: fewer than 2^31
    // quads, rows fewer than 2^31 bytes apart
    const int64_t quad_row = int64_t(g.nangles) * (g.cols + 2 * kColPad);
    const bool pad_fits = int64_t(g.rows + 2 * kRowPad) * quad_row < (int64_t(1) << 31) &&
                          quad_row * 16 < (int64_t(1) << 31);
    ap.bil_zflat = (pad_fits && voxel_ss == 1 && pu[0] == 0.0 && pw[0] == 0.0) ? 1 : 0;
    (ap.bil_zflat ? bil_fast : bil_slow)->push_back(t);
    for (int i = 0; i < 3; ++i) ap.src[i] = float(S[i]);

    // Forward-projection volume copy for this (d, a, b).
    int li = -1;
    for (size_t l = 0; l < p->layouts.size(); ++l)
      if (p->layouts[l].d == d && p->layouts[l].a == a && p->layouts[l].b == b) li = int(l);
    if (li < 0) {
      Layout L;
      L.d = d;
      L.a = a;
      L.b = b;
      L.n_d = shape[d];
      L.n_a = shape[a];
      L.n_b = shape[b];
      L.offset_elems = 0;
      p->layouts.push_back(L);
      li = int(p->layouts.size()) - 1;
    }
    ap.layout = li;

    // Column table (separable angles).
    if (separable) {
      for (int iu = 0; iu < g.cols; ++iu) {
        const double ut = double(iu - g.ou);
        const double den = e[0] + e[1] * ut;
        ColumnEntry& c = (*columns)[size_t(t) * g.cols + iu];
        c.Xa = float((ca[0] + ca[1] * ut) / den);
        c.ma = float((ma[0] + ma[1] * ut) / den);
        c.P = float((cb[0] + cb[1] * ut) / den);
        c.Q = float((mb[0] + mb[1] * ut) / den);
        c.R = float(cb[2] / den);
        c.S = float(mb[2] / den);
      }
    }
    ap.bp_general = (separable && b == 0) ? 0 : 1;
    if (ap.bp_general)
      gen_angles->push_back(t);
    else
      sep_angles->push_back(t);
    // Planes on which a column's rows lie closer than one voxel: the row step
    // q_b'(vt) = R + kt S is linear in the plane kt, so |R + kt S| < 1 on one
    // interval of planes; count the planes of [k_lo, k_hi] in it.
    if (!ap.bp_general) {
      const double k_lo = -double(anchor[d]), k_hi = double(shape[d] - 1 - anchor[d]);
      for (int iu = 0; iu < g.cols; ++iu) {
        const ColumnEntry& c = (*columns)[size_t(t) * g.cols + iu];
        double lo = k_lo, hi = k_hi;
        if (c.S != 0.0f) {
          const double a = (-1.0 - double(c.R)) / double(c.S), b = (1.0 - double(c.R)) / double(c.S);
          lo = std::max(lo, std::floor(std::min(a, b)) + 1.0);
          hi = std::min(hi, std::ceil(std::max(a, b)) - 1.0);
        } else if (!(std::fabs(double(c.R)) < 1.0)) {
          hi = lo - 1.0;
        }
        if (hi >= lo) fine_planes += hi - lo + 1.0;
        all_planes += k_hi - k_lo + 1.0;
      }
    }
  }

  int64_t off = 0;
  for (auto& L : p->layouts) {
    L.offset_elems = off;
    off += (L.elems() + 31) / 32 * 32;  // keep every copy 256-byte aligned
  }
  for (auto& ap : p->host_params) {
    const Layout& L = p->layouts[ap.layout];
    ap.ws_offset = L.offset_elems;
    ap.n_d = int(L.n_d);
    ap.n_a = int(L.n_a);
    ap.n_b = int(L.n_b);
    ap.o_d = anchor[L.d];
    ap.o_a = anchor[L.a];
    ap.o_b = anchor[L.b];
    ap.stride_a = int(L.n_b + 2 * kPad);
    ap.stride_d = int((L.n_a + 2 * kPad) * (L.n_b + 2 * kPad));
    ap.vs_d = float(vs[L.d]);
    ap.vs_a = float(vs[L.a]);
    ap.vs_b = float(vs[L.b]);
  }
  p->fp_workspace_elems = off;
  // At least a quarter of the separable work on rows finer than the voxels (a
  // supersampled or fine detector; about 0.6 % of it for the cone scans of the
  // benchmark): the matched backprojection takes the voxel-pair kernel's
  // fine-row variant.
  p->fine_rows = all_planes > 0.0 && fine_planes >= 0.25 * all_planes;
  // Detector region of a 16 x 8 x 16 voxel box at the anchor for each general
  // angle (its corners widened by one voxel along a and b, as the kernel
  // does; pixels from floor(min) to ceil(max) of their projections, an odd
  // stride): boxes nearer a cone's source project larger, hence the margin.
  p->gen_box_wide = true;
  for (int t : *gen_angles) {
    const AngleParams& ap = p->host_params[t];
    const double lo[3] = {-8.0, -4.0, -8.0}, hi[3] = {7.0, 3.0, 7.0};
    double umin = 1e300, umax = -1e300, vmin = 1e300, vmax = -1e300;
    bool ok = true;
    for (int c = 0; c < 8; ++c) {
      double P[3];
      for (int ax = 0; ax < 3; ++ax) {
        const double e = ax == ap.d ? 0.0 : 1.0;
        P[ax] = ((c >> ax) & 1) ? hi[ax] + e : lo[ax] - e;
      }
      const double nu = ap.pu[0] * P[0] + ap.pu[1] * P[1] + ap.pu[2] * P[2] + ap.pu[3];
      const double nv = ap.pv[0] * P[0] + ap.pv[1] * P[1] + ap.pv[2] * P[2] + ap.pv[3];
      const double nw = ap.pw[0] * P[0] + ap.pw[1] * P[1] + ap.pw[2] * P[2] + ap.pw[3];
      if (!(nw > 0.0)) {
        ok = false;
        break;
      }
      umin = std::min(umin, nu / nw);
      umax = std::max(umax, nu / nw);
      vmin = std::min(vmin, nv / nw);
      vmax = std::max(vmax, nv / nw);
    }
    const double nu = std::ceil(umax) - std::floor(umin) + 1.0;
    const double nv = std::ceil(vmax) - std::floor(vmin) + 1.0;
    if (!ok || 1.5 * (nu + 1.0) * (nv + 1.0) > 2048.0) {
      p->gen_box_wide = false;
      break;
    }
  }
  p->n_general_bp = int(gen_angles->size());
  // Separable angles grouped by their in-plane axis a (x first, then y): the
  // backprojector runs one pass per group, each with voxel runs along a.
  std::stable_partition(sep_angles->begin(), sep_angles->end(),
                        [&](int t) { return p->host_params[t].a == 2; });
  p->n_separable_bp = int(sep_angles->size());
  p->n_sep_ax = int(std::count_if(sep_angles->begin(), sep_angles->end(),
                                  [&](int t) { return p->host_params[t].a == 2; }));
  p->n_bil_fast = int(bil_fast->size());
  p->n_bil_slow = int(bil_slow->size());
  return std::string();
}

}  // namespace tsgb
