// Batched SIRT: one iteration of many independent reconstruction jobs as three
// kernel launches over all of them (padded volume copies, forward projection
// with the residual epilogue, backprojection with the update epilogue).
//
// There is no counterpart in the reference: tomosipo users loop SIRT in Python,
// one operator call and a few element-wise ops per step per job
// (README.md:150-163, notebooks/sirt_benchmark.py:116-136). Batching lets jobs
// of any size share each launch, so small jobs no longer leave SMs idle or pay
// per-call host overhead, and an iteration can be captured in one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "device_common.cuh"

struct tsgb_sirt_batch {
  int device = -1;
  tsgb::SirtBatchDev dev{};
  void* blob = nullptr;  // one device allocation holding all tables
};

namespace {

int bfail(int code, const std::string& msg) {
  tsgb::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" {

int tsgb_sirt_batch_create(const tsgb_sirt_job* jobs, int32_t n_jobs, tsgb_sirt_batch** out) {
  tsgb::set_last_error(std::string());
  if (!out || !jobs || n_jobs < 1 || n_jobs > 65536)
    return bfail(TSGB_ERR_INVALID, "need 1 to 65536 jobs and an output pointer");
  *out = nullptr;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return bfail(TSGB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));

  std::vector<tsgb::SirtJobDev> hj(n_jobs);
  std::vector<long long> fp_prefix(n_jobs + 1, 0), bp_prefix(n_jobs + 1, 0);
  std::vector<tsgb::LayoutSegDev> segs;
  long long max_seg = 0;
  for (int i = 0; i < n_jobs; ++i) {
    const tsgb_sirt_job& J = jobs[i];
    const tsgb_projector* p = J.projector;
    if (!p || !J.vol || !J.sino || !J.R || !J.C || !J.residual || !J.fp_workspace)
      return bfail(TSGB_ERR_INVALID, "job " + std::to_string(i) + " has a NULL pointer");
    if (p->device != dev)
      return bfail(TSGB_ERR_DEVICE, "job " + std::to_string(i) + " belongs to another device");
    if (p->n_general_bp > 0 || p->g.det_ss != 1)
      return bfail(TSGB_ERR_INVALID, "job " + std::to_string(i) +
                                         " has angles outside the separable backprojector "
                                         "(det_v not along z); run it with the plain operator");
    const tsgb::DeviceGeometry& g = p->g;
    tsgb::SirtJobDev& d = hj[i];
    d.params = p->d_params;
    d.columns = p->d_columns;
    d.sep_angles = p->d_sep_angles;
    d.n_sep = p->n_separable_bp;
    d.wide = (size_t)(g.rows + 2 * tsgb::kRowPad) * g.nangles * g.cols >= (size_t(1) << 31) ? 1 : 0;
    if (d.wide)
      return bfail(TSGB_ERR_INVALID, "job " + std::to_string(i) +
                                         " has a sinogram of 2^31 floats or more; run it with the "
                                         "plain operator");
    d.g = g;
    d.vol = J.vol;
    d.y = J.sino;
    d.R = J.R;
    d.C = J.C;
    d.res = J.residual;
    d.fp_ws = J.fp_workspace;
    // the job's forward tiles in its projector's order, one per angle pair
    d.fp_sched = tsgb::fp_schedule(p, (g.nangles + 1) / 2);
    d.bp_xb = (g.nx + tsgb::kBpTileX - 1) / tsgb::kBpTileX;
    d.bp_yb = (g.ny + tsgb::kBpTileY - 1) / tsgb::kBpTileY;
    d.bp_zb = (g.nz + tsgb::kBpRunZ - 1) / tsgb::kBpRunZ;
    fp_prefix[i + 1] = fp_prefix[i] + (long long)d.fp_sched.row_blocks *
                                          d.fp_sched.col_blocks * d.fp_sched.pairs;
    bp_prefix[i + 1] = bp_prefix[i] + (long long)d.bp_xb * d.bp_yb * d.bp_zb;
    const long long vstride[3] = {(long long)g.ny * g.nx, (long long)g.nx, 1};
    for (const auto& L : p->layouts) {
      tsgb::LayoutSegDev s;
      s.vol = J.vol;
      s.out = J.fp_workspace + L.offset_floats;
      s.n_d = L.n_d;
      s.n_a = L.n_a;
      s.n_b = L.n_b;
      s.s_d = vstride[L.d];
      s.s_a = vstride[L.a];
      s.s_b = vstride[L.b];
      segs.push_back(s);
      max_seg = std::max(max_seg, (long long)L.floats());
    }
  }
  if (segs.size() > 65535) return bfail(TSGB_ERR_INVALID, "too many volume copies in one batch");
  if (fp_prefix[n_jobs] >= (1LL << 31) || bp_prefix[n_jobs] >= (1LL << 31))
    return bfail(TSGB_ERR_INVALID, "batch too large for one launch");

  // One device allocation: jobs | fp prefix | bp prefix | segments.
  const size_t jb = sizeof(tsgb::SirtJobDev) * n_jobs;
  const size_t pb = sizeof(long long) * (n_jobs + 1);
  const size_t sb = sizeof(tsgb::LayoutSegDev) * std::max<size_t>(segs.size(), 1);
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t total = up(jb) + 2 * up(pb) + up(sb);
  std::vector<char> host(total, 0);
  std::copy_n(reinterpret_cast<const char*>(hj.data()), jb, host.data());
  std::copy_n(reinterpret_cast<const char*>(fp_prefix.data()), pb, host.data() + up(jb));
  std::copy_n(reinterpret_cast<const char*>(bp_prefix.data()), pb, host.data() + up(jb) + up(pb));
  if (!segs.empty())
    std::copy_n(reinterpret_cast<const char*>(segs.data()), sizeof(tsgb::LayoutSegDev) * segs.size(),
                host.data() + up(jb) + 2 * up(pb));

  tsgb_sirt_batch* b = new (std::nothrow) tsgb_sirt_batch();
  if (!b) return bfail(TSGB_ERR_INVALID, "host allocation failed");
  b->device = dev;
  e = cudaMalloc(&b->blob, total);
  if (e == cudaSuccess) e = cudaMemcpy(b->blob, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (b->blob) cudaFree(b->blob);
    delete b;
    return bfail(TSGB_ERR_CUDA, std::string("batch upload: ") + cudaGetErrorString(e));
  }
  char* base = static_cast<char*>(b->blob);
  b->dev.jobs = reinterpret_cast<tsgb::SirtJobDev*>(base);
  b->dev.fp_prefix = reinterpret_cast<long long*>(base + up(jb));
  b->dev.bp_prefix = reinterpret_cast<long long*>(base + up(jb) + up(pb));
  b->dev.segs = reinterpret_cast<tsgb::LayoutSegDev*>(base + up(jb) + 2 * up(pb));
  b->dev.n_jobs = n_jobs;
  b->dev.n_segs = int(segs.size());
  b->dev.fp_blocks = fp_prefix[n_jobs];
  b->dev.bp_blocks = bp_prefix[n_jobs];
  b->dev.seg_grid_x = std::max(1LL, std::min((max_seg + 255) / 256, 4096LL));
  *out = b;
  return TSGB_OK;
}

int tsgb_sirt_batch_iterate(tsgb_sirt_batch* b, int32_t iterations, void* stream) {
  tsgb::set_last_error(std::string());
  if (!b || iterations < 0) return bfail(TSGB_ERR_INVALID, "bad batch or iteration count");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != b->device) return bfail(TSGB_ERR_DEVICE, "current device differs from the batch's");
  for (int it = 0; it < iterations; ++it) {
    cudaError_t e = cudaError_t(tsgb::launch_sirt_fp_batch(b->dev, stream));
    if (e == cudaSuccess) e = cudaError_t(tsgb::launch_sirt_bp_batch(b->dev, stream));
    if (e != cudaSuccess) return bfail(TSGB_ERR_CUDA, std::string("batched SIRT launch: ") + cudaGetErrorString(e));
  }
  return TSGB_OK;
}

int tsgb_sirt_batch_destroy(tsgb_sirt_batch* b) {
  if (!b) return TSGB_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != b->device) cudaSetDevice(b->device);
  if (b->blob) cudaFree(b->blob);
  if (prev >= 0 && prev != b->device) cudaSetDevice(prev);
  delete b;
  return TSGB_OK;
}

}  // extern "C"
