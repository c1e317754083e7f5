// Internal types of the tomosipo_gb300 projector (not part of the C ABI).
//
// Coordinates. Kernels work in "anchored voxel coordinates": one unit per
// voxel along each axis, origin at the centre of voxel o = N / 2 (integer
// division), so voxel i sits at the integer i - o. Keeping the origin inside
// the volume keeps fp32 positions small (|q| <= N/2), which is what bounds
// their rounding error. Detector pixels are anchored the same way:
// pixel iu sits at iu - o_u with o_u = cols / 2.
//
// Discretisation (forward projection, Joseph's method). For each angle the
// host picks a dominant volume axis d (largest component of the central ray
// in voxel units) and two in-plane axes a and b. A ray is sampled on every
// voxel-centre plane k of axis d; its in-plane position there is
//   q_a(k) = X_a + kt * m_a,   q_b(k) = X_b + kt * m_b,   kt = k - o_d,
// where X is the ray's hit point on plane kt = 0 and m its slope per plane.
// The sample is the bilinear interpolation of the four voxels around
// (q_a, q_b) with zeros outside the volume. The ray sum is scaled by the
// world-space step between planes, W = |(vs_d, vs_a m_a, vs_b m_b)|.
// The matched backprojection is the exact transpose of this.
#pragma once

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "tomosipo_gb300.h"

namespace tsgb {

constexpr int kPad = 2;        // zero padding of the forward-projection volume copies
constexpr int kRowPad = 2;     // zero detector rows above and below the weighted sinogram
constexpr int kColPad = 2;     // zero detector columns left and right (bilinear BP copy)
constexpr int kMaxLayouts = 6; // axis permutations (d, a, b)

// Per-angle parameters, read uniformly by all threads of a block.
struct alignas(16) AngleParams {
  int d, a, b;       // volume axes (0 = z, 1 = y, 2 = x)
  int separable;     // det_v has no d or a component: column table is valid
  int layout;        // index of the padded volume copy used by the forward projector
  int bp_general;    // 1: backprojected by the general kernel (else separable kernel)
  int bil_zflat;     // projection's u numerator and denominator do not depend on z
  int pad1;
  // Ray coefficients, functions of anchored pixel coordinates (ut, vt):
  //   den = e0 + e1 ut + e2 vt,  X_a = (ca . [1,ut,vt]) / den,  m_a = (ma . [1,ut,vt]) / den
  // and the same for b. Parallel beams have den = 1.
  float e[4], ca[4], ma[4], cb[4], mb[4];
  // Projection of an anchored voxel position P = (z, y, x) onto the detector:
  //   ut = (pu . [P,1]) / (pw . [P,1]),  vt = (pv . [P,1]) / (pw . [P,1]),
  // normalised so that pw . [0,1] = 1.
  float pu[4], pv[4], pw[4];
  // Bilinear backprojection weight: parallel: bil_scale;
  // cone: bil_scale * |P - src|_world / (pw . [P,1])^3.
  float bil_scale;
  float src[3];      // source in anchored voxel coordinates (cone)
  // Addressing of this angle's padded forward-projection copy, laid out
  // [d][a][b] with b fastest: element (k along d, i along a, j along b;
  // unpadded indices) is at ws_offset + k * stride_d + (i + kPad) * stride_a + (j + kPad).
  long long ws_offset;
  int n_d, n_a, n_b;
  int o_d, o_a, o_b;
  int stride_d, stride_a;
  float vs_d, vs_a, vs_b;  // voxel size along d, a, b (world units)
  float pad2;
};

// Column table entry for separable angles, one per (angle, detector column):
//   q_a(kt) = X_a + kt m_a
//   q_b(kt, vt) = (P + vt R) + kt (Q + vt S)
struct alignas(16) ColumnEntry {
  float Xa, ma, P, Q;
  float R, S, pad0, pad1;
};

struct Layout {
  int d, a, b;
  int64_t n_d, n_a, n_b;   // unpadded extents
  // The forward workspace holds the copies as single voxels or, with the
  // tuning's fp_pair_layout, as pairs along b: element (k, i, j) =
  // (c[k][i][j], c[k][i][j+1]) of the padded copy c, so a bilinear sample is
  // two 8-byte loads. Offsets and sizes count elements; the workspace is sized
  // for pairs either way.
  int64_t offset_elems;   // offset of this copy in the forward workspace
  int64_t elems() const { return n_d * (n_a + 2 * kPad) * (n_b + 2 * kPad); }
};

struct DeviceGeometry {
  int kind;                 // TSGB_PARALLEL / TSGB_CONE
  int nz, ny, nx;           // volume shape
  int oz, oy, ox;           // voxel anchors (N / 2)
  int rows, cols, nangles;  // sinogram shape
  int ov, ou;               // pixel anchors
  float vs[3];              // voxel size (z, y, x), world units
  int det_ss, vox_ss;       // supersampling factors
};

// Forward-projection tile order over one chunk of angles (tsgb_tuning):
// groups of group_pairs angle pairs, each run over the detector patch by
// patch (patch_rows x patch_cols tiles), row tiles fastest inside a patch.
struct FpSchedule {
  int row_blocks, col_blocks, pairs;  // tiles along rows and columns; angle pairs
  int patch_rows, patch_cols, group_pairs;
};

}  // namespace tsgb

struct tsgb_projector {
  int device;
  tsgb::DeviceGeometry g;
  tsgb_tuning tuning;
  // Detector supersampling d > 1: `fine` projects onto the d-times finer
  // detector (forward projection and matched backprojection run there, with
  // binning / spreading passes; supersample.cu); this projector keeps the
  // coarse detector for shapes and the bilinear backprojection.
  int det_ss = 1;
  tsgb_projector* fine = nullptr;
  std::vector<tsgb::AngleParams> host_params;
  std::vector<tsgb::Layout> layouts;
  int64_t fp_workspace_elems = 0;  // 8-byte pair elements
  int n_general_bp = 0;         // angles handled by the general BP kernel
  int n_separable_bp = 0;       // angles handled by the separable BP kernel
  int n_sep_ax = 0;             // of those, the first n_sep_ax have a = x (the rest a = y)
  // On at least a quarter of the (separable angle, column, plane) triples the
  // detector rows lie closer than one voxel apart (|q_b step per row| < 1):
  // the matched backprojection then runs the voxel-pair kernel's fine-row
  // variant.
  bool fine_rows = false;
  // The general backprojector's voxel boxes may be 16 wide along x: the
  // detector region a 16 x 8 x 16 box at the volume's centre projects to, for
  // every general angle, stays within two thirds of the kernel's stage (else
  // boxes 8 wide, whose regions are about half as large).
  bool gen_box_wide = true;
  int n_bil_fast = 0;           // bilinear BP: angles for the z-flat kernel
  int n_bil_slow = 0;           // bilinear BP: angles for the general kernel
  tsgb::AngleParams* d_params = nullptr;
  tsgb::ColumnEntry* d_columns = nullptr;  // [nangles][cols]
  int* d_sep_angles = nullptr;             // angle ids for the separable BP kernel
  std::vector<int> host_sep_angles;        // the same lists on the host (angle ranges)
  std::vector<int> host_gen_angles;
  int* d_gen_angles = nullptr;             // angle ids for the general BP kernel
  int* d_bil_fast = nullptr;               // angle ids, bilinear z-flat kernel
  int* d_bil_slow = nullptr;               // angle ids, bilinear general kernel
};

namespace tsgb {

// One angle's detector frame and ray coefficients in anchored voxel
// coordinates (fp64), shared by build_plan and the no-allocation path.
struct AngleFrame {
  double U[3], V[3];   // det_u, det_v per voxel
  double Dc[3];        // centre of the anchored pixel (ov, ou)
  double S[3], R[3];   // source position (cone) / ray direction (parallel)
  int d, a, b;         // dominant axis, in-plane axes (b: the one det_v runs along)
  bool separable;      // det_v has no d or a component (then snapped to exact zeros)
  double e[3], ca[3], ma[3], cb[3], mb[3];  // ray coefficients over (1, ut, vt)
};

// Reduce row t of a projection's vectors ([src|ray, det_pos, det_v, det_u]);
// vs / origin: voxel size and the anchor voxel's centre (world). Returns "" or
// the error message (non-finite vectors, zero or parallel det_u / det_v, a
// zero ray direction, a degenerate cone frame).
std::string reduce_angle(const double* row, bool cone, const double vs[3], const double origin[3],
                         int rows, int cols, int ov, int ou, bool allow_separable, int t,
                         AngleFrame* f);

// Host-side construction of the per-angle tables in fp64 (plan.cpp). Fills
// p->g, p->host_params, p->layouts and the column table; returns an empty
// string on success, else the error message.
std::string build_plan(const tsgb_volume_desc* vol, const tsgb_projection_desc* proj,
                       int voxel_ss, int det_ss, tsgb_projector* p,
                       std::vector<ColumnEntry>* columns,
                       std::vector<int>* sep_angles, std::vector<int>* gen_angles,
                       std::vector<int>* bil_fast, std::vector<int>* bil_slow);

// Schedule of `pairs` angle pairs under the projector's tuning (fp.cu).
FpSchedule fp_schedule(const tsgb_projector* p, int pairs);
// Angles per forward-projection launch (fp.cu).
long long fp_angle_chunk(const DeviceGeometry& g);
// Default tuning of a new projector whose plan is built (fp.cu).
tsgb_tuning default_tuning(const tsgb_projector* p);

// FDK backprojection of a weighted, ramp-filtered sinogram (cone beams whose
// angles all take the z-flat bilinear path; workspace as the bilinear BP's).
int launch_bp_fdk(const tsgb_projector* p, float* vol, const float* sino, const float* angle_w,
                  bool additive, float* workspace, void* stream);

// Detector supersampling passes between p's detector and p->fine's (supersample.cu).
int launch_ss_bin(const tsgb_projector* p, const float* fine, float* coarse, bool additive,
                  void* stream);
int launch_ss_expand(const tsgb_projector* p, const float* coarse, float* fine, void* stream);

// Sets the calling thread's message returned by tsgb_last_error (capi.cu).
void set_last_error(const std::string& msg);

// SIRT epilogue of the forward projection: instead of a sinogram it writes
// res = W * (R * (y - A x)) in the backprojector's row-pair layout, where W is
// each ray's plane step (see bp_weight_kernel). res holds
// 2 * (rows + 2 kRowPad) * nangles * cols floats whose padding rows are zero;
// zlayout: column-major pairs (bp_weight_z_kernel), else row-major.
struct FpSirt {
  const float* y;  // measured sinogram
  const float* R;  // per-ray weights (sinogram-shaped)
  float* res;
  int zlayout;
};

// Multi-job launches of batched SIRT: one launch covers many small jobs, block
// b running block b - start[j] of job j (start[j] <= b < start[j + 1]). The job
// descriptors travel as __grid_constant__ kernel arguments.
constexpr int kMaxMultiJobs = 48;
// Batched projections share multi-job launches in groups of items whose
// per-item workspaces (volume copies, weighted sinograms) fit this budget: the
// launches pay off for items too small to fill the GPU alone.
constexpr int64_t kBatchWorkspaceBudget = int64_t(2) << 30;
inline int64_t batch_group(int64_t n, int64_t item_bytes) {
  if (item_bytes <= 0) return 1;
  const int64_t fit = kBatchWorkspaceBudget / item_bytes;
  return std::max<int64_t>(1, std::min<int64_t>({n, int64_t(kMaxMultiJobs), fit}));
}

struct FpMultiJob {
  const AngleParams* params;
  const ColumnEntry* columns;
  const void* ws;  // the job's padded volume copies
  DeviceGeometry g;
  FpSchedule sched;
  FpSirt sirt;     // SIRT launches: where the residual goes
  float* sino;     // plain launches: the job's sinogram (= or += when additive)
  int additive;
};
struct FpMulti {
  int n;
  long long start[kMaxMultiJobs + 1];
  FpMultiJob job[kMaxMultiJobs];
};

struct BpMultiJob {
  const AngleParams* params;
  const ColumnEntry* columns;
  const int* angles;  // this pass's angle ids
  const float* pairs; // the job's residual (row-major row pairs)
  float* vol;
  const float* C;
  float* scratch;     // first pass's sum (nullptr: none)
  DeviceGeometry g;
  int n_angles, mode; // mode: 2 = keep the sum in scratch, 3 = apply the update
  int gx, gy;         // the job's own grid (x, y); z = blocks / (gx * gy)
};
struct BpMulti {
  int n;
  long long start[kMaxMultiJobs + 1];
  BpMultiJob job[kMaxMultiJobs];
};
// kernel arguments are limited to 32764 bytes
static_assert(sizeof(FpMulti) <= 32764 && sizeof(BpMulti) <= 32764, "multi-job tables too large");

// The padded volume copies of a forward projection, no rays (fp.cu).
int launch_fp_copies(const tsgb_projector* p, const float* vol, float* workspace, void* stream);
// Whether a job's SIRT forward projection fits a multi-job launch (one angle
// chunk), its block count, and the multi-job launch itself (fp.cu).
bool fp_multi_eligible(const tsgb_projector* p);
long long fp_blocks(const tsgb_projector* p);
// sirt: each job writes its SIRT residual; else its sinogram.
int launch_fp_multi(const FpMulti& m, bool pair_layout, void* stream, bool sirt = true);
// Forward projection of n stacked volumes of one projector on multi-job
// launches (fp_multi_eligible, no supersampling), `group` items per launch
// (<= kMaxMultiJobs): item k's volume copies at workspace + (k % group) *
// item_bytes (fp.cu).
int launch_fp_batch(const tsgb_projector* p, const float* vol, float* sino, int64_t n,
                    bool additive, char* workspace, int64_t item_bytes, int group, void* stream);
// Blocks of one voxel-pair backprojection pass of a job (gx, gy set), and
// the multi-job launch of that pass over several jobs (bp.cu).
long long bp_sep_blocks(const tsgb_projector* p, bool a_is_x, int* gx, int* gy);
int launch_bp_sep_multi(const BpMulti& m, bool a_is_x, void* stream);
// Whether a projector's batched matched backprojection can run on multi-job
// launches (voxel-pair kernel, separable angles only, 32-bit offsets, no
// supersampling or fine-row variant), and that batched backprojection:
// `group` items per launch (<= kMaxMultiJobs), item k's weighted sinogram at
// workspace + (k % group) * item_bytes (item_bytes >= bp_pairs_bytes) (bp.cu).
bool bp_batch_multi_eligible(const tsgb_projector* p);
int launch_bp_matched_batch(const tsgb_projector* p, float* vol, const float* sino, int64_t n,
                            bool additive, char* workspace, int64_t item_bytes, int group,
                            void* stream);

// The matched backprojector of det_v-along-z angles is the z-lane kernel
// (bp_zlane.cu, column-major weighted sinogram) unless the tuning picks the
// voxel-pair kernel (bp.cu, row-major), the volume's (y, x) plane is too
// large for the z-lane grid (fewer than 2^32 voxel columns keep it below 2^31
// blocks for every shape, which hold at least 8 columns per block), or the
// detector rows are mostly finer than the voxels (fine_rows: the voxel-pair
// kernel has a fast path for that).
inline bool bp_uses_zlane(const tsgb_projector* p) {
  return p->tuning.bp_kernel == 1 && !p->fine_rows &&
         int64_t(p->g.nx) * p->g.ny < (int64_t(1) << 32);
}
inline int zlane_shape(const tsgb_projector* p) { return p->tuning.bp_shape; }

// Bytes of the matched backprojection's weighted sinogram (either layout),
// rounded up to 256; the z-lane kernel's [y][x][z] scratch volume follows it.
int64_t bp_pairs_bytes(const DeviceGeometry& g);
int64_t bp_volume_bytes(const DeviceGeometry& g);

// Column-major row-pair weighted sinogram (float pairs) of angles
// angle_begin .. angle_end - 1 (bp_zlane.cu).
int launch_bp_weight_z(const tsgb_projector* p, const float* sino, float* sinoz, int angle_begin,
                       int angle_end, void* stream);
// Both z-lane passes over the separable angle lists (offsets into
// p->d_sep_angles) into the [y][x][z] scratch volt, then vol (=, +=, SIRT)
// from it (out_mode 0 / 1 / 2; C for SIRT). False if there are no such angles.
bool launch_bp_zlane_separable(const tsgb_projector* p, int off_x, int n_ax, int off_y, int n_ay,
                               const float* sinoz, float* volt, float* vol, int out_mode,
                               const float* C, void* stream);

// Kernel launchers (fp.cu, bp.cu). All return cudaGetLastError() as int.
// With `sirt` the forward projection writes the SIRT residual instead of sino.
// angle_begin / angle_end: project only these angles (their sinogram slices;
// -1 = all); copies_ready: the workspace already holds this volume's copies.
int launch_fp(const tsgb_projector* p, const float* vol, float* sino, bool additive,
              float* workspace, void* stream, const FpSirt* sirt = nullptr, int angle_begin = 0,
              int angle_end = -1, bool copies_ready = false);
int launch_bp_matched(const tsgb_projector* p, float* vol, const float* sino, bool additive,
                      float* workspace, void* stream, int angle_begin = 0, int angle_end = -1);
int launch_bp_bilinear(const tsgb_projector* p, float* vol, const float* sino, bool additive,
                       float* workspace, void* stream);

// SIRT update x += C * A^T(res) from a residual written by launch_fp's SIRT
// epilogue (separable angles only), rounded as the plain recipe's x += C * bp.
// scratch: a volume-sized buffer (the forward workspace is free by then).
int launch_bp_sirt(const tsgb_projector* p, float* vol, const float* C, const float* res,
                   float* scratch, void* stream);
constexpr int kBpRunZ = 16;  // voxels along z per matched-backprojection thread
constexpr int kBpTileX = 32, kBpTileY = 4, kFpTileRows = 32, kFpTileCols = 8;

}  // namespace tsgb
