// extern "C" entry points of libtomosipo_gb300 (declared in include/tomosipo_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>

#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tsgb_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(TSGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void free_device(tsgb_projector* p) {
  if (p->d_params) cudaFree(p->d_params);
  if (p->d_columns) cudaFree(p->d_columns);
  if (p->d_sep_angles) cudaFree(p->d_sep_angles);
  if (p->d_gen_angles) cudaFree(p->d_gen_angles);
  if (p->d_bil_fast) cudaFree(p->d_bil_fast);
  if (p->d_bil_slow) cudaFree(p->d_bil_slow);
  p->d_bil_fast = nullptr;
  p->d_bil_slow = nullptr;
  p->d_params = nullptr;
  p->d_columns = nullptr;
  p->d_sep_angles = nullptr;
  p->d_gen_angles = nullptr;
}

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& src) {
  const size_t bytes = (src.empty() ? 1 : src.size()) * sizeof(T);
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), bytes);
  if (e != cudaSuccess) return e;
  if (!src.empty()) e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

int check_device(const tsgb_projector* p) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != p->device)
    return fail(TSGB_ERR_DEVICE, "current CUDA device " + std::to_string(dev) +
                                     " differs from the projector's device " +
                                     std::to_string(p->device));
  return TSGB_OK;
}

}  // namespace

namespace tsgb {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace tsgb

extern "C" {

int tsgb_projector_create(const tsgb_volume_desc* vol, const tsgb_projection_desc* proj,
                          int32_t voxel_supersampling, int32_t detector_supersampling,
                          tsgb_projector** out) {
  g_last_error.clear();
  if (!out) return fail(TSGB_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (detector_supersampling < 1 || detector_supersampling > 16)
    return fail(TSGB_ERR_INVALID, "supersampling factors must lie in [1, 16]");
  tsgb_projector* p = new (std::nothrow) tsgb_projector();
  if (!p) return fail(TSGB_ERR_INVALID, "host allocation failed");
  std::vector<tsgb::ColumnEntry> columns;
  std::vector<int> sep, gen, bfast, bslow;
  std::string err = tsgb::build_plan(vol, proj, voxel_supersampling, 1, p, &columns, &sep, &gen,
                                     &bfast, &bslow);
  if (!err.empty()) {
    delete p;
    return fail(TSGB_ERR_INVALID, err);
  }
  for (const auto& L : p->layouts)
    if (L.elems() >= (int64_t(1) << 31)) {
      delete p;
      return fail(TSGB_ERR_INVALID, "volume too large for 32-bit indexing of one padded copy");
    }
  if (p->g.nz > 65535 || p->g.ny > 2000000 || p->g.nx > 2000000 || p->g.rows > 4 * 65535 ||
      p->g.cols > 8 * 65535) {
    delete p;
    return fail(TSGB_ERR_INVALID,
                "volume z extent must be <= 65535, y and x extents <= 2000000, detector rows "
                "<= 262140 and columns <= 524280");
  }
  p->tuning = tsgb::default_tuning(p);
  if (detector_supersampling > 1) {
    // the d-times finer detector: same centre, pixel vectors divided by d
    const int d = detector_supersampling;
    std::vector<double> fine(size_t(proj->num_angles) * 12);
    for (size_t i = 0; i < fine.size(); ++i)
      fine[i] = proj->vectors[i] / ((i % 12) >= 6 ? double(d) : 1.0);
    tsgb_projection_desc fd = *proj;
    fd.det_shape[0] = proj->det_shape[0] * d;
    fd.det_shape[1] = proj->det_shape[1] * d;
    fd.vectors = fine.data();
    int rc = tsgb_projector_create(vol, &fd, voxel_supersampling, 1, &p->fine);
    if (rc != TSGB_OK) {
      delete p;
      return fail(rc, "supersampled detector: " + g_last_error);
    }
    p->det_ss = d;
    p->g.det_ss = d;
  }
  cudaError_t e = cudaGetDevice(&p->device);
  if (e == cudaSuccess) e = upload(&p->d_params, p->host_params);
  if (e == cudaSuccess) e = upload(&p->d_columns, columns);
  p->host_sep_angles = sep;
  p->host_gen_angles = gen;
  if (e == cudaSuccess) e = upload(&p->d_sep_angles, sep);
  if (e == cudaSuccess) e = upload(&p->d_gen_angles, gen);
  if (e == cudaSuccess) e = upload(&p->d_bil_fast, bfast);
  if (e == cudaSuccess) e = upload(&p->d_bil_slow, bslow);
  if (e != cudaSuccess) {
    free_device(p);
    if (p->fine) tsgb_projector_destroy(p->fine);
    delete p;
    return cuda_fail(e, "projector upload");
  }
  *out = p;
  return TSGB_OK;
}

int tsgb_projector_destroy(tsgb_projector* p) {
  g_last_error.clear();
  if (!p) return TSGB_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != p->device) cudaSetDevice(p->device);
  free_device(p);
  if (prev >= 0 && prev != p->device) cudaSetDevice(prev);
  if (p->fine) tsgb_projector_destroy(p->fine);
  delete p;
  return TSGB_OK;
}

namespace {

// Bytes of p->fine's sinogram, rounded up to 256 (the workspace part that
// precedes p->fine's own workspace when the detector is supersampled).
int64_t fine_sino_bytes(const tsgb_projector* p) {
  const tsgb::DeviceGeometry& f = p->fine->g;
  return (int64_t(f.rows) * f.nangles * f.cols * int64_t(sizeof(float)) + 255) / 256 * 256;
}

}  // namespace

int64_t tsgb_fp_workspace_bytes(const tsgb_projector* p) {
  if (!p) return fail(TSGB_ERR_INVALID, "projector is NULL");
  if (p->fine) return fine_sino_bytes(p) + tsgb_fp_workspace_bytes(p->fine);
  return p->fp_workspace_elems * int64_t(2 * sizeof(float));  // pairs of floats
}

int64_t tsgb_bp_workspace_bytes(const tsgb_projector* p, int32_t bp_kind) {
  if (!p) return fail(TSGB_ERR_INVALID, "projector is NULL");
  if (bp_kind == TSGB_BP_BILINEAR)
    // quad copy of the padded sinogram: four floats per element
    return p->n_bil_fast > 0 ? int64_t(p->g.rows + 2 * tsgb::kRowPad) * p->g.nangles *
                                   (p->g.cols + 2 * tsgb::kColPad) * int64_t(4 * sizeof(float))
                             : 0;
  if (bp_kind != TSGB_BP_MATCHED) return fail(TSGB_ERR_INVALID, "unknown bp_kind");
  if (p->fine) return fine_sino_bytes(p) + tsgb_bp_workspace_bytes(p->fine, bp_kind);
  // row-pair weighted sinogram (two floats per pixel, kRowPad padding rows),
  // then the z-lane kernel's [y][x][z] scratch volume (either kernel may run)
  return tsgb::bp_pairs_bytes(p->g) +
         (p->n_separable_bp > 0 ? tsgb::bp_volume_bytes(p->g) : int64_t(0));
}

int tsgb_projector_shapes(const tsgb_projector* p, int64_t vol_shape[3], int64_t sino_shape[3]) {
  if (!p) return fail(TSGB_ERR_INVALID, "projector is NULL");
  if (vol_shape) {
    vol_shape[0] = p->g.nz;
    vol_shape[1] = p->g.ny;
    vol_shape[2] = p->g.nx;
  }
  if (sino_shape) {
    sino_shape[0] = p->g.rows;
    sino_shape[1] = p->g.nangles;
    sino_shape[2] = p->g.cols;
  }
  return TSGB_OK;
}

int tsgb_direct_fp(tsgb_projector* p, const float* vol, float* sino, int32_t additive,
                   void* workspace, int64_t workspace_bytes, void* stream) {
  g_last_error.clear();
  if (!p || !vol || !sino) return fail(TSGB_ERR_INVALID, "NULL projector or data pointer");
  const int64_t need = tsgb_fp_workspace_bytes(p);
  if (need > 0 && (!workspace || workspace_bytes < need))
    return fail(TSGB_ERR_WORKSPACE, "forward projection needs " + std::to_string(need) +
                                        " bytes of workspace");
  int rc = check_device(p);
  if (rc != TSGB_OK) return rc;
  cudaError_t e;
  if (p->fine) {
    // project onto the finer detector, then bin d x d blocks into sino
    float* fine_sino = static_cast<float*>(workspace);
    float* fine_ws = reinterpret_cast<float*>(static_cast<char*>(workspace) + fine_sino_bytes(p));
    e = cudaError_t(tsgb::launch_fp(p->fine, vol, fine_sino, false, fine_ws, stream));
    if (e == cudaSuccess) e = cudaError_t(tsgb::launch_ss_bin(p, fine_sino, sino, additive != 0, stream));
  } else {
    e = cudaError_t(
        tsgb::launch_fp(p, vol, sino, additive != 0, static_cast<float*>(workspace), stream));
  }
  if (e != cudaSuccess) return cuda_fail(e, "forward projection launch");
  return TSGB_OK;
}

int tsgb_direct_bp(tsgb_projector* p, float* vol, const float* sino, int32_t additive,
                   int32_t bp_kind, void* workspace, int64_t workspace_bytes, void* stream) {
  g_last_error.clear();
  if (!p || !vol || !sino) return fail(TSGB_ERR_INVALID, "NULL projector or data pointer");
  if (bp_kind != TSGB_BP_MATCHED && bp_kind != TSGB_BP_BILINEAR)
    return fail(TSGB_ERR_INVALID, "unknown bp_kind");
  const int64_t need = tsgb_bp_workspace_bytes(p, bp_kind);
  if (need > 0 && (!workspace || workspace_bytes < need))
    return fail(TSGB_ERR_WORKSPACE,
                "backprojection needs " + std::to_string(need) + " bytes of workspace");
  int rc = check_device(p);
  if (rc != TSGB_OK) return rc;
  cudaError_t e;
  if (bp_kind == TSGB_BP_MATCHED && p->fine) {
    // the transpose of the binning: spread each pixel / d^2 over its block,
    // then the finer detector's matched backprojection
    float* fine_sino = static_cast<float*>(workspace);
    float* fine_ws = reinterpret_cast<float*>(static_cast<char*>(workspace) + fine_sino_bytes(p));
    e = cudaError_t(tsgb::launch_ss_expand(p, sino, fine_sino, stream));
    if (e == cudaSuccess)
      e = cudaError_t(tsgb::launch_bp_matched(p->fine, vol, fine_sino, additive != 0, fine_ws, stream));
  } else if (bp_kind == TSGB_BP_MATCHED)
    e = cudaError_t(tsgb::launch_bp_matched(p, vol, sino, additive != 0,
                                            static_cast<float*>(workspace), stream));
  else
    e = cudaError_t(tsgb::launch_bp_bilinear(p, vol, sino, additive != 0,
                                             static_cast<float*>(workspace), stream));
  if (e != cudaSuccess) return cuda_fail(e, "backprojection launch");
  return TSGB_OK;
}

int64_t tsgb_fp_batch_workspace_bytes(const tsgb_projector* p, int64_t n) {
  const int64_t one = tsgb_fp_workspace_bytes(p);
  if (one <= 0 || n <= 1 || p->fine || !tsgb::fp_multi_eligible(p)) return one;
  const int64_t group = tsgb::batch_group(n, one);
  return group > 1 ? group * one : one;
}

int tsgb_direct_fp_batch(tsgb_projector* p, const float* vol, float* sino, int64_t n,
                         int32_t additive, void* workspace, int64_t workspace_bytes,
                         void* stream) {
  g_last_error.clear();
  if (!p || !vol || !sino || n < 0) return fail(TSGB_ERR_INVALID, "NULL projector or data pointer");
  const size_t vol_elems = size_t(p->g.nz) * p->g.ny * p->g.nx;
  const size_t sino_elems = size_t(p->g.rows) * p->g.nangles * p->g.cols;
  // multi-job launches when the workspace holds the volume copies of every
  // item of a group (tsgb_fp_batch_workspace_bytes); else one after another
  const int64_t one = tsgb_fp_workspace_bytes(p);
  const int64_t group = one > 0 && workspace ? std::min<int64_t>({n, int64_t(tsgb::kMaxMultiJobs),
                                                                 workspace_bytes / one})
                                             : 0;
  if (group > 1 && !p->fine && tsgb::fp_multi_eligible(p)) {
    int rc = check_device(p);
    if (rc != TSGB_OK) return rc;
    cudaError_t e = cudaError_t(tsgb::launch_fp_batch(p, vol, sino, n, additive != 0,
                                                      static_cast<char*>(workspace), one,
                                                      int(group), stream));
    if (e != cudaSuccess) return cuda_fail(e, "batched forward projection launch");
    return TSGB_OK;
  }
  // one workspace serves every item: the projections run one after another on
  // the stream
  for (int64_t i = 0; i < n; ++i) {
    const int rc = tsgb_direct_fp(p, vol + i * vol_elems, sino + i * sino_elems, additive,
                                  workspace, workspace_bytes, stream);
    if (rc != TSGB_OK) return rc;
  }
  return TSGB_OK;
}

int64_t tsgb_bp_batch_workspace_bytes(const tsgb_projector* p, int64_t n, int32_t bp_kind) {
  const int64_t one = tsgb_bp_workspace_bytes(p, bp_kind);
  if (one < 0 || n <= 1 || bp_kind != TSGB_BP_MATCHED || !tsgb::bp_batch_multi_eligible(p))
    return one;
  const int64_t item = tsgb::bp_pairs_bytes(p->g), group = tsgb::batch_group(n, item);
  return group > 1 ? std::max<int64_t>(one, group * item) : one;
}

int tsgb_direct_bp_batch(tsgb_projector* p, float* vol, const float* sino, int64_t n,
                         int32_t additive, int32_t bp_kind, void* workspace,
                         int64_t workspace_bytes, void* stream) {
  g_last_error.clear();
  if (!p || !vol || !sino || n < 0) return fail(TSGB_ERR_INVALID, "NULL projector or data pointer");
  const size_t vol_elems = size_t(p->g.nz) * p->g.ny * p->g.nx;
  const size_t sino_elems = size_t(p->g.rows) * p->g.nangles * p->g.cols;
  // multi-job launches when the workspace holds a weighted sinogram per item
  // of a group (tsgb_bp_batch_workspace_bytes); else one item after another
  const int64_t item = tsgb::bp_pairs_bytes(p->g);
  const int64_t group = workspace ? std::min<int64_t>({n, int64_t(tsgb::kMaxMultiJobs),
                                                       workspace_bytes / item})
                                  : 0;
  if (group > 1 && bp_kind == TSGB_BP_MATCHED && tsgb::bp_batch_multi_eligible(p)) {
    int rc = check_device(p);
    if (rc != TSGB_OK) return rc;
    cudaError_t e = cudaError_t(tsgb::launch_bp_matched_batch(
        p, vol, sino, n, additive != 0, static_cast<char*>(workspace), item, int(group), stream));
    if (e != cudaSuccess) return cuda_fail(e, "batched backprojection launch");
    return TSGB_OK;
  }
  for (int64_t i = 0; i < n; ++i) {
    const int rc = tsgb_direct_bp(p, vol + i * vol_elems, sino + i * sino_elems, additive, bp_kind,
                                  workspace, workspace_bytes, stream);
    if (rc != TSGB_OK) return rc;
  }
  return TSGB_OK;
}

int tsgb_direct_fp_angles(tsgb_projector* p, const float* vol, float* sino, int32_t additive,
                          int64_t angle_begin, int64_t angle_end, int32_t copies_ready,
                          void* workspace, int64_t workspace_bytes, void* stream) {
  g_last_error.clear();
  if (!p || !vol || !sino) return fail(TSGB_ERR_INVALID, "NULL projector or data pointer");
  if (p->fine) return fail(TSGB_ERR_INVALID, "angle ranges need detector supersampling 1");
  if (angle_begin < 0 || angle_end > p->g.nangles || angle_begin >= angle_end)
    return fail(TSGB_ERR_INVALID, "angle range outside 0 .. num_angles");
  const int64_t need = tsgb_fp_workspace_bytes(p);
  if (need > 0 && (!workspace || workspace_bytes < need))
    return fail(TSGB_ERR_WORKSPACE, "forward projection needs " + std::to_string(need) +
                                        " bytes of workspace");
  int rc = check_device(p);
  if (rc != TSGB_OK) return rc;
  cudaError_t e = cudaError_t(tsgb::launch_fp(p, vol, sino, additive != 0,
                                              static_cast<float*>(workspace), stream, nullptr,
                                              int(angle_begin), int(angle_end), copies_ready != 0));
  if (e != cudaSuccess) return cuda_fail(e, "forward projection launch");
  return TSGB_OK;
}

int tsgb_direct_bp_angles(tsgb_projector* p, float* vol, const float* sino, int32_t additive,
                          int64_t angle_begin, int64_t angle_end, void* workspace,
                          int64_t workspace_bytes, void* stream) {
  g_last_error.clear();
  if (!p || !vol || !sino) return fail(TSGB_ERR_INVALID, "NULL projector or data pointer");
  if (p->fine) return fail(TSGB_ERR_INVALID, "angle ranges need detector supersampling 1");
  if (angle_begin < 0 || angle_end > p->g.nangles || angle_begin >= angle_end)
    return fail(TSGB_ERR_INVALID, "angle range outside 0 .. num_angles");
  const int64_t need = tsgb_bp_workspace_bytes(p, TSGB_BP_MATCHED);
  if (need > 0 && (!workspace || workspace_bytes < need))
    return fail(TSGB_ERR_WORKSPACE,
                "backprojection needs " + std::to_string(need) + " bytes of workspace");
  int rc = check_device(p);
  if (rc != TSGB_OK) return rc;
  cudaError_t e = cudaError_t(tsgb::launch_bp_matched(p, vol, sino, additive != 0,
                                                      static_cast<float*>(workspace), stream,
                                                      int(angle_begin), int(angle_end)));
  if (e != cudaSuccess) return cuda_fail(e, "backprojection launch");
  return TSGB_OK;
}

int tsgb_copy_sino_angles(void* dst, const void* src, int64_t rows, int64_t num_angles,
                          int64_t cols, int64_t angle_begin, int64_t angle_end, void* stream) {
  g_last_error.clear();
  if (!dst || !src || rows < 1 || cols < 1 || angle_begin < 0 || angle_end > num_angles ||
      angle_begin >= angle_end)
    return fail(TSGB_ERR_INVALID, "bad sinogram copy arguments");
  const size_t pitch = size_t(num_angles) * cols * sizeof(float);
  const size_t off = size_t(angle_begin) * cols * sizeof(float);
  cudaError_t e = cudaMemcpy2DAsync(static_cast<char*>(dst) + off, pitch,
                                    static_cast<const char*>(src) + off, pitch,
                                    size_t(angle_end - angle_begin) * cols * sizeof(float),
                                    size_t(rows), cudaMemcpyDefault,
                                    static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "sinogram copy");
  return TSGB_OK;
}

int tsgb_fdk_backproject(tsgb_projector* p, float* vol, const float* filtered, const float* angle_weights,
                         int32_t additive, void* workspace, int64_t workspace_bytes, void* stream) {
  g_last_error.clear();
  if (!p || !vol || !filtered || !angle_weights)
    return fail(TSGB_ERR_INVALID, "NULL projector or data pointer");
  if (p->g.kind != TSGB_CONE) return fail(TSGB_ERR_INVALID, "FDK needs a cone beam");
  const int64_t need = tsgb_bp_workspace_bytes(p, TSGB_BP_BILINEAR);
  if (!workspace || workspace_bytes < need)
    return fail(TSGB_ERR_WORKSPACE, "FDK needs " + std::to_string(need) + " bytes of workspace");
  int rc = check_device(p);
  if (rc != TSGB_OK) return rc;
  cudaError_t e = cudaError_t(tsgb::launch_bp_fdk(p, vol, filtered, angle_weights, additive != 0,
                                                  static_cast<float*>(workspace), stream));
  if (e != cudaSuccess) return cuda_fail(e, "FDK backprojection launch");
  return TSGB_OK;
}

int tsgb_projector_stats(const tsgb_projector* p, int64_t* out, int32_t n) {
  if (!p || !out || n < 0 || n > 8) return fail(TSGB_ERR_INVALID, "bad stats arguments");
  // FP and matched BP run on the finer detector when it is supersampled, plus
  // one binning / spreading launch
  const tsgb_projector* f = p->fine ? p->fine : p;
  const int64_t extra = p->fine ? 1 : 0;
  const int64_t chunks = (f->g.nangles + 65534) / 65535;
  const int64_t chunk = tsgb::fp_angle_chunk(f->g);
  const int64_t fp_launches =
      int64_t(f->layouts.size()) + (f->g.nangles + chunk - 1) / chunk + extra;
  // weight pass, one launch per separable pass, the z-lane kernel's transpose
  // out of its scratch, the general kernel
  const int64_t bp_launches = chunks + (f->n_sep_ax > 0 ? 1 : 0) +
                              (f->n_separable_bp - f->n_sep_ax > 0 ? 1 : 0) +
                              (tsgb::bp_uses_zlane(f) && f->n_separable_bp > 0 ? 1 : 0) +
                              ((f->n_general_bp > 0 || f->n_separable_bp == 0) ? 1 : 0) + extra;
  const int64_t vals[8] = {int64_t(f->layouts.size()),
                           f->n_separable_bp,
                           f->n_general_bp,
                           fp_launches,
                           bp_launches,
                           (p->n_bil_fast > 0 ? 2 : 0) +
                               ((p->n_bil_slow > 0 || p->n_bil_fast == 0) ? 1 : 0),
                           tsgb_fp_workspace_bytes(p),
                           tsgb_bp_workspace_bytes(p, TSGB_BP_MATCHED)};
  for (int i = 0; i < n; ++i) out[i] = vals[i];
  return TSGB_OK;
}

int tsgb_projector_get_tuning(const tsgb_projector* p, tsgb_tuning* out) {
  g_last_error.clear();
  if (!p || !out) return fail(TSGB_ERR_INVALID, "projector or out is NULL");
  *out = p->fine ? p->fine->tuning : p->tuning;  // the projector that runs the FP
  return TSGB_OK;
}

int tsgb_projector_set_tuning(tsgb_projector* p, const tsgb_tuning* t) {
  g_last_error.clear();
  if (!p || !t) return fail(TSGB_ERR_INVALID, "projector or tuning is NULL");
  if (t->fp_patch_rows < 1 || t->fp_patch_cols < 1 || t->fp_group_pairs < 1)
    return fail(TSGB_ERR_INVALID, "tuning values must be >= 1");
  if (t->fp_pair_layout != 0 && t->fp_pair_layout != 1)
    return fail(TSGB_ERR_INVALID, "fp_pair_layout must be 0 or 1");
  if (t->bp_kernel != 0 && t->bp_kernel != 1) return fail(TSGB_ERR_INVALID, "bp_kernel must be 0 or 1");
  if (t->bp_shape < 0 || t->bp_shape > 6) return fail(TSGB_ERR_INVALID, "bp_shape must lie in 0 .. 6");
  if (t->bp_general != 0 && t->bp_general != 1)
    return fail(TSGB_ERR_INVALID, "bp_general must be 0 or 1");
  if (t->reserved != 0) return fail(TSGB_ERR_INVALID, "reserved tuning fields must be 0");
  // the projector that runs the FP and the matched BP
  (p->fine ? p->fine : p)->tuning = *t;
  return TSGB_OK;
}

const char* tsgb_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
