// tsgb_direct_fp_noalloc: a forward projection that allocates no device memory.
//
// Who needs it: code that cannot call cudaMalloc on its hot path -- for example a
// projector called from inside another framework's custom-call hook, whose memory
// belongs to that framework's allocator, or a real-time acquisition loop that has
// a fixed device-memory budget and must not trigger an allocation (which can
// synchronise the device) while it runs. Such callers pass only the geometry,
// their input volume and their output sinogram.
//
// How: the scratch the forward projector needs (zero-padded volume copies, one per
// axis permutation) and the per-angle parameters live in file-scope
// `static __device__` arrays of fixed size. Their limits:
//   * padded copies: at most kScratchFloats = 16,777,216 floats (64 MiB), i.e.
//     sum over the permutations used of n_d * (n_a + 4) * (n_b + 4) floats
//     (a circular cone or parallel scan of a 160^3 volume needs two copies,
//     2 * 160 * 164 * 164 = 8.6 M floats);
//   * angles: at most kMaxAngles = 4096.
// Larger requests are rejected with TSGB_ERR_INVALID and a message.
//
// Every call shares the arrays and leaves the previous call's contents behind:
// each call rewrites every scratch float it reads (padding included) and uploads
// its own angle parameters, so nothing stale is used, but calls whose work
// overlaps on the GPU (different streams, or different host threads without
// ordering) race on the arrays. Serialize them on one stream.
//
// Set-up: the first call on each device resolves the arrays' device addresses
// with cudaGetSymbolAddress (the array names in host code are only host-side
// stand-ins) with that device current. Make that first call before any stream
// capture. The arrays occupy device memory on every GPU where this module is
// loaded (on the first use of this entry point under CUDA's default lazy module
// loading, at library load with CUDA_MODULE_LOADING=EAGER) until the process exits.
//
// The per-angle parameters reach the device as kernel arguments (chunks of
// kParamChunk angles, written into the static parameter array by a small copy
// kernel on the caller's stream), so a call issues no host-to-device memcpy and
// keeps no host buffer that a later call could overwrite before it is read.
//
// The arithmetic is the forward projector of fp.cu (Joseph's method on the
// dominant axis of each angle, bilinear in-plane, scaled by the plane step), with
// every ray's coefficients computed from the per-angle parameters. The per-angle
// reduction (frame, dominant axis, ray coefficients, and the checks that reject
// degenerate detectors) is plan.cpp's reduce_angle, the same function the
// regular projector's planner uses.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "device_common.cuh"

namespace {

constexpr long long kScratchFloats = 1LL << 24;  // 64 MiB of padded volume copies
constexpr int kMaxAngles = 4096;
constexpr int kMaxDevices = 64;
constexpr int kRows = 32;  // threads along detector rows (one warp)
constexpr int kCols = 8;   // warps along detector columns
constexpr float kMaxSlope = 64.0f;
constexpr int kParamChunk = 64;  // angles per parameter-copy launch (16 KiB of arguments)

static __device__ __align__(256) float g_scratch[kScratchFloats];
static __device__ __align__(256) tsgb::AngleParams g_params[kMaxAngles];

std::mutex g_mutex;                           // guards the host staging buffer and set-up
tsgb::AngleParams g_host_params[kMaxAngles];  // host staging of the per-angle parameters
void* g_scratch_ptr[kMaxDevices] = {};  // device addresses, resolved once per device
void* g_params_ptr[kMaxDevices] = {};

// One chunk of per-angle parameters, passed by value as a kernel argument.
struct ParamChunk {
  tsgb::AngleParams p[kParamChunk];
};

// Copies `count` parameter entries from the launch's arguments to dst.
__global__ void noalloc_params_kernel(const __grid_constant__ ParamChunk chunk, int count,
                                      tsgb::AngleParams* __restrict__ dst) {
  static_assert(sizeof(tsgb::AngleParams) % sizeof(int4) == 0, "16-byte words");
  const int4* src = reinterpret_cast<const int4*>(chunk.p);
  int4* out = reinterpret_cast<int4*>(dst);
  const int words = count * int(sizeof(tsgb::AngleParams) / sizeof(int4));
  for (int i = threadIdx.x; i < words; i += blockDim.x) out[i] = src[i];
}

int fail(int code, const std::string& msg) {
  tsgb::set_last_error(msg);  // read back through tsgb_last_error()
  return code;
}

__global__ void noalloc_layout_kernel(const float* __restrict__ vol, float* __restrict__ out,
                                      long long n_d, long long n_a, long long n_b, long long s_d,
                                      long long s_a, long long s_b) {
  const long long n_ap = n_a + 2 * tsgb::kPad, n_bp = n_b + 2 * tsgb::kPad;
  const long long total = n_d * n_ap * n_bp;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long jp = idx % n_bp, rest = idx / n_bp;
    const long long ip = rest % n_ap, k = rest / n_ap;
    const long long i = ip - tsgb::kPad, j = jp - tsgb::kPad;
    float v = 0.0f;
    if (i >= 0 && i < n_a && j >= 0 && j < n_b) v = __ldg(vol + k * s_d + i * s_a + j * s_b);
    out[idx] = v;
  }
}

__device__ __forceinline__ void narrow(float X, float m, float lo, float hi, float& klo,
                                       float& khi) {
  if (m != 0.0f) {
    const float inv = 1.0f / m;
    const float t1 = (lo - X) * inv, t2 = (hi - X) * inv;
    klo = fmaxf(klo, fminf(t1, t2));
    khi = fminf(khi, fmaxf(t1, t2));
  } else if (!(X > lo && X < hi)) {
    klo = 1.0f;
    khi = 0.0f;
  }
}

__global__ void __launch_bounds__(kRows* kCols)
    noalloc_fp_kernel(const tsgb::AngleParams* __restrict__ params,
                      const float* __restrict__ scratch, float* __restrict__ sino,
                      tsgb::DeviceGeometry g, int additive) {
  const int iv = blockIdx.x * kRows + threadIdx.x;
  const int iu = blockIdx.y * kCols + threadIdx.y;
  const int theta = blockIdx.z;
  if (iu >= g.cols || iv >= g.rows) return;
  const tsgb::AngleParams& ap = params[theta];
  const tsgb::Ray r = tsgb::ray_general(ap, float(iu - g.ou), float(iv - g.ov));
  float total = 0.0f;
  if (tsgb::finite_ray(r) && fabsf(r.ma) <= kMaxSlope && fabsf(r.mb) <= kMaxSlope) {
    float klo = float(-ap.o_d), khi = float(ap.n_d - 1 - ap.o_d);
    narrow(r.Xa, r.ma, float(-1 - ap.o_a), float(ap.n_a - ap.o_a), klo, khi);
    narrow(r.Xb, r.mb, float(-1 - ap.o_b), float(ap.n_b - ap.o_b), klo, khi);
    if (klo <= khi) {
      const float* base = scratch + ap.ws_offset + (long long)ap.o_d * ap.stride_d +
                          (long long)(ap.o_a + tsgb::kPad) * ap.stride_a + (ap.o_b + tsgb::kPad);
      float acc = 0.0f;
      for (int k = (int)ceilf(klo); k <= (int)floorf(khi); ++k) {
        const float qa = fmaf(float(k), r.ma, r.Xa), qb = fmaf(float(k), r.mb, r.Xb);
        const float fa0 = floorf(qa), fb0 = floorf(qb);
        const float fa = qa - fa0, fb = qb - fb0;
        const float* p = base + (k * ap.stride_d + (int)fa0 * ap.stride_a + (int)fb0);
        const float left = fmaf(fb, __ldg(p + 1) - __ldg(p), __ldg(p));
        const float right = fmaf(fb, __ldg(p + ap.stride_a + 1) - __ldg(p + ap.stride_a),
                                 __ldg(p + ap.stride_a));
        acc += fmaf(fa, right - left, left);
      }
      total = acc * tsgb::ray_step(ap, r);
    }
  }
  float* out = sino + ((size_t)iv * g.nangles + theta) * g.cols + iu;
  if (additive)
    *out += total;
  else
    *out = total;
}

// Per-angle parameters (fp64 -> fp32) of the forward projector, written into
// g_host_params; returns "" or an error message. Layout offsets go to lay_*.
std::string plan_angles(const tsgb_volume_desc* vol, const tsgb_projection_desc* proj,
                        tsgb::DeviceGeometry* g, int lay_dab[6][3], long long lay_offset[6],
                        int* n_layouts) {
  const bool cone = proj->kind == TSGB_CONE;
  const int shape[3] = {g->nz, g->ny, g->nx};
  const int anchor[3] = {g->oz, g->oy, g->ox};
  double vs[3], origin[3];
  for (int i = 0; i < 3; ++i) {
    vs[i] = vol->size[i] / double(vol->shape[i]);
    g->vs[i] = float(vs[i]);
    origin[i] = vol->pos[i] - 0.5 * vol->size[i] + (anchor[i] + 0.5) * vs[i];
  }
  *n_layouts = 0;
  long long used = 0;
  for (int t = 0; t < g->nangles; ++t) {
    tsgb::AngleFrame f;
    const std::string err = tsgb::reduce_angle(proj->vectors + 12 * (size_t)t, cone, vs, origin,
                                               g->rows, g->cols, g->ov, g->ou, true, t, &f);
    if (!err.empty()) return err;
    const int d = f.d, a = f.a, b = f.b;
    tsgb::AngleParams ap{};
    ap.d = d;
    ap.a = a;
    ap.b = b;
    for (int j = 0; j < 3; ++j) {
      ap.e[j] = float(f.e[j]);
      ap.ca[j] = float(f.ca[j]);
      ap.ma[j] = float(f.ma[j]);
      ap.cb[j] = float(f.cb[j]);
      ap.mb[j] = float(f.mb[j]);
    }
    int li = -1;
    for (int l = 0; l < *n_layouts; ++l)
      if (lay_dab[l][0] == d && lay_dab[l][1] == a && lay_dab[l][2] == b) li = l;
    if (li < 0) {
      li = (*n_layouts)++;
      lay_dab[li][0] = d;
      lay_dab[li][1] = a;
      lay_dab[li][2] = b;
      lay_offset[li] = used;
      const long long floats =
          (long long)shape[d] * (shape[a] + 2 * tsgb::kPad) * (shape[b] + 2 * tsgb::kPad);
      used += (floats + 63) / 64 * 64;
      if (used > kScratchFloats)
        return "volume needs " + std::to_string(used) +
               " floats of padded copies; the no-allocation path holds at most " +
               std::to_string(kScratchFloats) + " (64 MiB)";
    }
    ap.layout = li;
    ap.ws_offset = lay_offset[li];
    ap.n_d = shape[d];
    ap.n_a = shape[a];
    ap.n_b = shape[b];
    ap.o_d = anchor[d];
    ap.o_a = anchor[a];
    ap.o_b = anchor[b];
    ap.stride_a = shape[b] + 2 * tsgb::kPad;
    ap.stride_d = (shape[a] + 2 * tsgb::kPad) * (shape[b] + 2 * tsgb::kPad);
    ap.vs_d = float(vs[d]);
    ap.vs_a = float(vs[a]);
    ap.vs_b = float(vs[b]);
    g_host_params[t] = ap;
  }
  return std::string();
}

}  // namespace

extern "C" int tsgb_direct_fp_noalloc(const tsgb_volume_desc* vol,
                                      const tsgb_projection_desc* proj, const float* vol_in,
                                      float* sino_out, int32_t additive, void* stream_) {
  tsgb::set_last_error(std::string());
  if (!vol || !proj || !proj->vectors || !vol_in || !sino_out)
    return fail(TSGB_ERR_INVALID, "NULL descriptor or data pointer");
  if (proj->kind != TSGB_PARALLEL && proj->kind != TSGB_CONE)
    return fail(TSGB_ERR_INVALID, "projection kind must be TSGB_PARALLEL or TSGB_CONE");
  if (proj->num_angles < 1 || proj->num_angles > kMaxAngles)
    return fail(TSGB_ERR_INVALID, "the no-allocation path takes 1 to " +
                                      std::to_string(kMaxAngles) + " angles");
  for (int i = 0; i < 3; ++i)
    if (vol->shape[i] < 1 || vol->shape[i] > 65535 || !(vol->size[i] > 0) ||
        !std::isfinite(vol->size[i]) || !std::isfinite(vol->pos[i]))
      return fail(TSGB_ERR_INVALID, "volume shape or size out of range");
  if (proj->det_shape[0] < 1 || proj->det_shape[1] < 1 || proj->det_shape[0] > 4 * 65535 ||
      proj->det_shape[1] > 8 * 65535)
    return fail(TSGB_ERR_INVALID, "detector shape out of range");

  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(TSGB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(TSGB_ERR_DEVICE, "device index out of range");

  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {  // once per device, with that device current
    void* s = nullptr;
    void* q = nullptr;
    e = cudaGetSymbolAddress(&s, g_scratch);
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_params);
    if (e != cudaSuccess)
      return fail(TSGB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_params_ptr[dev] = q;
    g_scratch_ptr[dev] = s;
  }

  tsgb::DeviceGeometry g{};
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
  g.det_ss = 1;
  g.vox_ss = 1;
  int lay_dab[6][3];
  long long lay_offset[6];
  int n_layouts = 0;
  std::string err = plan_angles(vol, proj, &g, lay_dab, lay_offset, &n_layouts);
  if (!err.empty()) return fail(TSGB_ERR_INVALID, err);

  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  float* scratch = static_cast<float*>(g_scratch_ptr[dev]);
  tsgb::AngleParams* params = static_cast<tsgb::AngleParams*>(g_params_ptr[dev]);
  // Parameters as kernel arguments: the launch copies each chunk, so
  // g_host_params is free again as soon as the launch returns.
  for (int t0 = 0; t0 < g.nangles; t0 += kParamChunk) {
    const int count = std::min(kParamChunk, g.nangles - t0);
    ParamChunk chunk;
    std::memcpy(chunk.p, g_host_params + t0, sizeof(tsgb::AngleParams) * count);
    noalloc_params_kernel<<<1, 256, 0, stream>>>(chunk, count, params + t0);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(TSGB_ERR_CUDA, std::string("parameter upload: ") + cudaGetErrorString(e));
  const int shape[3] = {g.nz, g.ny, g.nx};
  const long long vstride[3] = {(long long)g.ny * g.nx, (long long)g.nx, 1};
  for (int l = 0; l < n_layouts; ++l) {
    const int d = lay_dab[l][0], a = lay_dab[l][1], b = lay_dab[l][2];
    const long long total =
        (long long)shape[d] * (shape[a] + 2 * tsgb::kPad) * (shape[b] + 2 * tsgb::kPad);
    const long long blocks = (total + 255) / 256;
    noalloc_layout_kernel<<<int(blocks < 152LL * 64 ? blocks : 152LL * 64), 256, 0, stream>>>(
        vol_in, scratch + lay_offset[l], shape[d], shape[a], shape[b], vstride[d], vstride[a],
        vstride[b]);
  }
  const dim3 block(kRows, kCols);
  const dim3 grid((g.rows + kRows - 1) / kRows, (g.cols + kCols - 1) / kCols, g.nangles);
  noalloc_fp_kernel<<<grid, block, 0, stream>>>(params, scratch, sino_out, g, additive ? 1 : 0);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(TSGB_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return TSGB_OK;
}
