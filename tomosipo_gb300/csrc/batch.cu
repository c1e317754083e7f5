// Batched SIRT: many independent reconstruction jobs advanced together.
//
// There is no counterpart in the reference: tomosipo users loop SIRT in Python,
// one operator call and a few element-wise ops per step per job
// (README.md:150-163, notebooks/sirt_benchmark.py:116-136).
//
// Each job runs the projector's own kernels with fused SIRT epilogues: the
// forward projection writes the residual W * R * (y - A x) straight into the
// backprojector's row-pair layout, and the backprojection applies
// x += C * A^T(res), so one iteration of one job is its padded volume copies
// plus two kernels, with no element-wise passes.
//
// Small jobs (at most 128^3 voxels, voxel-pair backprojector, no tilted
// detectors) are grouped, up to kMaxMultiJobs at a time, into multi-job
// launches: one forward launch and one launch per backprojection pass cover
// the whole group, each block running one tile of one job exactly as that
// job's own launch would (the job descriptors travel as __grid_constant__
// kernel arguments, so the per-job kernels keep their registers). A small
// job's backprojection alone fills a fraction of the SMs for a time set by its
// angle count, whatever its volume; in a group its blocks queue behind the
// others' and the SMs stay busy. Larger jobs keep their own launches.
//
// Work units (a large job, or a group of small ones) are spread over a small
// pool of streams (largest first, round robin), forked from and joined back
// into the caller's stream, so units run beside each other. Under stream
// capture the fork and join become a CUDA graph with one branch per stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "tsgb_internal.h"

namespace {

// Streams per batch: at most the default number of hardware queues
// (CUDA_DEVICE_MAX_CONNECTIONS = 8), so streams never share a queue.
constexpr int kMaxStreams = 8;
// Jobs of at most this many voxels (128^3) join multi-job launches.
constexpr long long kMultiMaxVoxels = 1LL << 21;

// A stream's unit of work: one job on its own launches, or a group of small
// jobs of one copy layout on multi-job launches.
struct Unit {
  std::vector<int> jobs;  // indices into the batch's (sorted) jobs
  bool multi = false;
  bool pair_layout = false;
  double work = 0.0;
};

bool multi_eligible(const tsgb_projector* p) {
  const tsgb::DeviceGeometry& g = p->g;
  int gx = 0, gy = 0;
  return (long long)g.nz * g.ny * g.nx <= kMultiMaxVoxels && !tsgb::bp_uses_zlane(p) &&
         p->n_general_bp == 0 && tsgb::fp_multi_eligible(p) &&
         tsgb::bp_sep_blocks(p, true, &gx, &gy) >= 0;
}

int bfail(int code, const std::string& msg) {
  tsgb::set_last_error(msg);
  return code;
}

}  // namespace

struct tsgb_sirt_batch {
  int device = -1;
  std::vector<tsgb_sirt_job> jobs;  // largest first
  std::vector<int> index;           // jobs[k] is the caller's job index[k]
  std::vector<Unit> units;          // largest first; unit u runs on stream u % streams
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
};

namespace {

void release(tsgb_sirt_batch* b) {
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  b->streams.clear();
  b->joins.clear();
  b->fork = nullptr;
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

  std::vector<double> work(n_jobs);
  for (int i = 0; i < n_jobs; ++i) {
    const tsgb_sirt_job& J = jobs[i];
    const tsgb_projector* p = J.projector;
    if (!p || !J.vol || !J.sino || !J.R || !J.C || !J.residual || !J.fp_workspace)
      return bfail(TSGB_ERR_INVALID, "job " + std::to_string(i) + " has a NULL pointer");
    if (p->device != dev)
      return bfail(TSGB_ERR_DEVICE, "job " + std::to_string(i) + " belongs to another device");
    if (p->fine)
      return bfail(TSGB_ERR_INVALID, "job " + std::to_string(i) +
                                         " uses detector supersampling; run it with the plain "
                                         "operator");
    const tsgb::DeviceGeometry& g = p->g;
    work[i] = double(g.nz) * g.ny * g.nx * g.nangles;
  }
  tsgb_sirt_batch* b = new (std::nothrow) tsgb_sirt_batch();
  if (!b) return bfail(TSGB_ERR_INVALID, "host allocation failed");
  b->device = dev;
  std::vector<int> order(n_jobs);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return work[a] > work[c]; });
  for (int i : order) {
    b->jobs.push_back(jobs[i]);
    b->index.push_back(i);
  }
  // units: each large job alone; the small ones by copy layout, in groups of
  // at most kMaxMultiJobs (a group of one is a plain unit)
  std::vector<int> small[2];
  for (int k = 0; k < n_jobs; ++k) {
    const tsgb_projector* p = b->jobs[k].projector;
    if (multi_eligible(p))
      small[p->tuning.fp_pair_layout ? 1 : 0].push_back(k);
    else
      b->units.push_back(Unit{{k}, false, false, work[order[k]]});
  }
  for (int layout = 0; layout < 2; ++layout) {
    const int n = int(small[layout].size());
    const int groups = (n + tsgb::kMaxMultiJobs - 1) / tsgb::kMaxMultiJobs;
    for (int q = 0; q < groups; ++q) {
      Unit u;
      u.multi = true;
      u.pair_layout = layout == 1;
      for (int k = q; k < n; k += groups) {  // groups of near-equal size and work
        u.jobs.push_back(small[layout][k]);
        u.work += work[order[small[layout][k]]];
      }
      if (u.jobs.size() == 1) u.multi = false;
      b->units.push_back(u);
    }
  }
  std::stable_sort(b->units.begin(), b->units.end(),
                   [](const Unit& a, const Unit& c) { return a.work > c.work; });

  const int n_streams = std::min(int(b->units.size()), kMaxStreams);
  e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (int k = 0; k < n_streams && e == cudaSuccess; ++k) {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) b->streams.push_back(s);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) b->joins.push_back(ev);
  }
  if (e != cudaSuccess) {
    release(b);
    delete b;
    return bfail(TSGB_ERR_CUDA, std::string("batch streams: ") + cudaGetErrorString(e));
  }
  *out = b;
  return TSGB_OK;
}

}  // extern "C"

namespace {

// One SIRT iteration of job J on its own launches.
cudaError_t iterate_job(const tsgb_sirt_job& J, cudaStream_t s) {
  const tsgb::FpSirt sirt{J.sino, J.R, J.residual, tsgb::bp_uses_zlane(J.projector) ? 1 : 0};
  cudaError_t e = cudaError_t(tsgb::launch_fp(J.projector, J.vol, nullptr, false, J.fp_workspace, s, &sirt));
  // the forward workspace is free once the residual is written: it holds the
  // first backprojection pass's sum
  if (e == cudaSuccess)
    e = cudaError_t(tsgb::launch_bp_sirt(J.projector, J.vol, J.C, J.residual, J.fp_workspace, s));
  return e;
}

// One SIRT iteration of the small jobs `members` on multi-job launches: each
// job's volume copies, one forward launch, then one launch per backprojection
// pass; every job's arithmetic is that of iterate_job.
cudaError_t iterate_group(const std::vector<const tsgb_sirt_job*>& members, bool pair_layout,
                          cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  tsgb::FpMulti fm{};
  for (const tsgb_sirt_job* J : members) {
    const tsgb_projector* p = J->projector;
    e = cudaError_t(tsgb::launch_fp_copies(p, J->vol, J->fp_workspace, s));
    if (e != cudaSuccess) return e;
    tsgb::FpMultiJob& F = fm.job[fm.n];
    F.params = p->d_params;
    F.columns = p->d_columns;
    F.ws = J->fp_workspace;
    F.g = p->g;
    F.sched = tsgb::fp_schedule(p, (p->g.nangles + 1) / 2);
    F.sirt = tsgb::FpSirt{J->sino, J->R, J->residual, 0};
    fm.start[fm.n + 1] = fm.start[fm.n] + tsgb::fp_blocks(p);
    ++fm.n;
  }
  e = cudaError_t(tsgb::launch_fp_multi(fm, pair_layout, s));
  // Backprojection: the pass along x, then the pass along y (which adds the
  // first pass's sum from the forward workspace); a job with angles in one
  // pass only applies its update there. Jobs with more angles (longer blocks)
  // go first.
  std::vector<const tsgb_sirt_job*> by_angles(members);
  std::stable_sort(by_angles.begin(), by_angles.end(),
                   [](const tsgb_sirt_job* a, const tsgb_sirt_job* c) {
                     return a->projector->g.nangles > c->projector->g.nangles;
                   });
  for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass) {
    const bool a_is_x = pass == 0;
    tsgb::BpMulti bm{};
    for (const tsgb_sirt_job* J : by_angles) {
      const tsgb_projector* p = J->projector;
      const int n_ax = p->n_sep_ax, n_ay = p->n_separable_bp - p->n_sep_ax;
      const int n = a_is_x ? n_ax : n_ay;
      if (n == 0) continue;
      const bool both = n_ax > 0 && n_ay > 0;
      tsgb::BpMultiJob& B = bm.job[bm.n];
      B.params = p->d_params;
      B.columns = p->d_columns;
      B.angles = p->d_sep_angles + (a_is_x ? 0 : n_ax);
      B.n_angles = n;
      B.pairs = J->residual;
      B.vol = J->vol;
      B.C = J->C;
      B.scratch = both ? J->fp_workspace : nullptr;
      B.mode = (a_is_x && both) ? 2 : 3;
      B.g = p->g;
      bm.start[bm.n + 1] = bm.start[bm.n] + tsgb::bp_sep_blocks(p, a_is_x, &B.gx, &B.gy);
      ++bm.n;
    }
    e = cudaError_t(tsgb::launch_bp_sep_multi(bm, a_is_x, s));
  }
  return e;
}

// Iterations count[k] of the batch's job k (its sorted order), forked from and
// joined back into `stream`.
int iterate_counts(tsgb_sirt_batch* b, const std::vector<int>& count, cudaStream_t stream) {
  int iterations = 0;
  for (int c : count) iterations = std::max(iterations, c);
  if (iterations == 0) return TSGB_OK;
  const int K = int(b->streams.size());
  cudaError_t e = cudaEventRecord(b->fork, stream);
  for (int k = 0; k < K && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->streams[k], b->fork, 0);
  // Iteration-major submission keeps the streams' queues interleaved; a
  // job's iterations stay in order on its stream, units never wait for each
  // other.
  std::vector<const tsgb_sirt_job*> members;
  for (int it = 0; it < iterations && e == cudaSuccess; ++it) {
    for (size_t u = 0; u < b->units.size() && e == cudaSuccess; ++u) {
      const Unit& U = b->units[u];
      cudaStream_t s = b->streams[u % K];
      members.clear();
      for (int k : U.jobs)
        if (it < count[k]) members.push_back(&b->jobs[k]);
      if (members.empty()) continue;
      if (U.multi && members.size() > 1)
        e = iterate_group(members, U.pair_layout, s);
      else
        for (size_t m = 0; m < members.size() && e == cudaSuccess; ++m)
          e = iterate_job(*members[m], s);
    }
  }
  for (int k = 0; k < K && e == cudaSuccess; ++k) {
    e = cudaEventRecord(b->joins[k], b->streams[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, b->joins[k], 0);
  }
  if (e != cudaSuccess) return bfail(TSGB_ERR_CUDA, std::string("batched SIRT launch: ") + cudaGetErrorString(e));
  return TSGB_OK;
}

int check_batch_device(const tsgb_sirt_batch* b) {
  int dev = -1;
  cudaGetDevice(&dev);
  return dev == b->device ? TSGB_OK
                          : bfail(TSGB_ERR_DEVICE, "current device differs from the batch's");
}

}  // namespace

extern "C" {

int tsgb_sirt_batch_iterate(tsgb_sirt_batch* b, int32_t iterations, void* stream) {
  tsgb::set_last_error(std::string());
  if (!b || iterations < 0) return bfail(TSGB_ERR_INVALID, "bad batch or iteration count");
  const int rc = check_batch_device(b);
  if (rc != TSGB_OK) return rc;
  return iterate_counts(b, std::vector<int>(b->jobs.size(), iterations),
                        static_cast<cudaStream_t>(stream));
}

int tsgb_sirt_batch_iterate_jobs(tsgb_sirt_batch* b, const int32_t* iterations, void* stream) {
  tsgb::set_last_error(std::string());
  if (!b || !iterations) return bfail(TSGB_ERR_INVALID, "bad batch or iteration counts");
  const int rc = check_batch_device(b);
  if (rc != TSGB_OK) return rc;
  std::vector<int> count(b->jobs.size());
  for (size_t k = 0; k < count.size(); ++k) {
    count[k] = iterations[b->index[k]];
    if (count[k] < 0) return bfail(TSGB_ERR_INVALID, "negative iteration count");
  }
  return iterate_counts(b, count, static_cast<cudaStream_t>(stream));
}

int tsgb_sirt_batch_destroy(tsgb_sirt_batch* b) {
  if (!b) return TSGB_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != b->device) cudaSetDevice(b->device);
  for (cudaStream_t s : b->streams) cudaStreamSynchronize(s);
  release(b);
  if (prev >= 0 && prev != b->device) cudaSetDevice(prev);
  delete b;
  return TSGB_OK;
}

}  // extern "C"
