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
// plus two kernels, with no element-wise passes. Jobs are spread over a small
// pool of streams (largest first, round robin), forked from and joined back
// into the caller's stream: small jobs run beside large ones and fill the SMs
// a single small launch would leave idle. Under stream capture the fork and
// join become a CUDA graph with one branch per stream.
//
// One fused launch over all jobs was the earlier design; it read each job's
// geometry from a device table, and the registers that cost (values the
// per-job kernels take from the parameter bank) made large jobs ~15 % slower
// than running them alone, which outweighed the gain on small jobs.
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

int bfail(int code, const std::string& msg) {
  tsgb::set_last_error(msg);
  return code;
}

}  // namespace

struct tsgb_sirt_batch {
  int device = -1;
  std::vector<tsgb_sirt_job> jobs;  // largest first
  std::vector<int> index;           // jobs[k] is the caller's job index[k]
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

  const int n_streams = std::min(n_jobs, kMaxStreams);
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
  // job's iterations stay in order on its stream, jobs never wait for each
  // other.
  for (int it = 0; it < iterations && e == cudaSuccess; ++it) {
    for (size_t i = 0; i < b->jobs.size() && e == cudaSuccess; ++i) {
      if (it >= count[i]) continue;
      const tsgb_sirt_job& J = b->jobs[i];
      cudaStream_t s = b->streams[i % K];
      const tsgb::FpSirt sirt{J.sino, J.R, J.residual, tsgb::bp_uses_zlane(J.projector) ? 1 : 0};
      e = cudaError_t(tsgb::launch_fp(J.projector, J.vol, nullptr, false, J.fp_workspace, s, &sirt));
      // the forward workspace is free once the residual is written: it holds
      // the first backprojection pass's sum
      if (e == cudaSuccess)
        e = cudaError_t(tsgb::launch_bp_sirt(J.projector, J.vol, J.C, J.residual, J.fp_workspace, s));
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
