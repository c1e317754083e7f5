/*
 * tomosipo_gb300 -- C ABI of the GB300 (sm_103a) tomographic projector.
 *
 * This library replaces the link layer of tomosipo, ``tomosipo/astra.py``,
 * which hands projection work to ASTRA's ``cuda3d`` projector. Every entry
 * point takes plain pointers and sizes; no C++ or PyTorch types cross the ABI.
 * Entry points return TSGB_OK (0) or a negative error code and never throw;
 * ``tsgb_last_error`` gives a message for the calling thread's last failure.
 *
 * Layouts (tomosipo's, ``tomosipo/links/base.py:21-31``):
 *   volume   : float32 [Nz][Ny][Nx], C-contiguous, x fastest
 *   sinogram : float32 [rows][num_angles][cols], C-contiguous, u fastest
 * All device pointers must be on the device the projector was created on.
 * Work is queued on ``stream`` (a cudaStream_t; NULL = legacy default
 * stream) and is asynchronous with respect to the host.
 */
#ifndef TOMOSIPO_GB300_H
#define TOMOSIPO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TSGB_OK 0
#define TSGB_ERR_INVALID (-1)   /* bad argument, shape or geometry */
#define TSGB_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define TSGB_ERR_WORKSPACE (-3) /* workspace missing or too small */
#define TSGB_ERR_DEVICE (-4)    /* current device differs from the projector's */

#define TSGB_PARALLEL 0 /* rows of ``vectors`` start with a ray direction */
#define TSGB_CONE 1     /* rows of ``vectors`` start with a source position */

#define TSGB_BP_MATCHED 0  /* exact transpose of the forward projector */
#define TSGB_BP_BILINEAR 1 /* voxel-driven, bilinear detector interpolation */

/* Axis-aligned volume: the form ``ts.operator`` reduces every volume to
 * (``tomosipo/Operator.py:11-60``) before it builds a projector. */
typedef struct {
  int64_t shape[3]; /* voxels (z, y, x) */
  double pos[3];    /* centre (z, y, x) */
  double size[3];   /* physical size (z, y, x) */
} tsgb_volume_desc;

/* Projection geometry in vector form (``pg.to_vec()``). Row ``t`` of
 * ``vectors`` (num_angles x 12 doubles) is
 *   [ src_pos or ray_dir (z,y,x), det_pos (z,y,x), det_v (z,y,x), det_u (z,y,x) ]
 * with det_pos the detector centre and det_v / det_u one pixel up / across
 * (``tomosipo/geometry/cone_vec.py``, ``parallel_vec.py``). */
typedef struct {
  int32_t kind;         /* TSGB_PARALLEL or TSGB_CONE */
  int32_t reserved;
  int64_t det_shape[2]; /* rows, cols */
  int64_t num_angles;
  const double* vectors;
} tsgb_projection_desc;

typedef struct tsgb_projector tsgb_projector;

/* Build a projector for one volume/projection geometry pair on the current
 * CUDA device. Replaces ``create_astra_projector`` (tomosipo/astra.py:80-98).
 * Supersampling factors must be >= 1 (1 = none): detector supersampling d
 * averages d*d rays per pixel in the forward projection (and its transpose);
 * voxel supersampling d averages d*d*d points per voxel in the bilinear
 * backprojection. Allocates the per-angle tables on the device. */
int tsgb_projector_create(const tsgb_volume_desc* vol,
                          const tsgb_projection_desc* proj,
                          int32_t voxel_supersampling,
                          int32_t detector_supersampling,
                          tsgb_projector** out);

/* Free a projector (ASTRA: astra.projector3d.delete; the reference leaves it
 * to garbage collection). Synchronises the projector's device. */
int tsgb_projector_destroy(tsgb_projector* p);

/* Bytes of device workspace ``tsgb_direct_fp`` / ``tsgb_direct_bp`` need
 * (0 if none); a negative error code for a NULL projector or an unknown
 * bp_kind. No counterpart in the reference (ASTRA allocates internally). */
int64_t tsgb_fp_workspace_bytes(const tsgb_projector* p);
int64_t tsgb_bp_workspace_bytes(const tsgb_projector* p, int32_t bp_kind);

/* Forward projection sino = A(vol), or sino += A(vol) when ``additive``.
 * Replaces ``direct_fp`` -> ``astra.experimental.direct_FPBP3D(projector,
 * vol, proj, MODE_SET|MODE_ADD, "FP")`` (tomosipo/astra.py:104-184). */
int tsgb_direct_fp(tsgb_projector* p, const float* vol, float* sino,
                   int32_t additive, void* workspace, int64_t workspace_bytes,
                   void* stream);

/* Backprojection vol = A^T(sino) (bp_kind TSGB_BP_MATCHED) or its
 * voxel-driven bilinear approximation (TSGB_BP_BILINEAR); vol += ... when
 * ``additive``. Replaces ``direct_bp`` -> ``direct_FPBP3D(..., "BP")``
 * (tomosipo/astra.py:187-217). */
int tsgb_direct_bp(tsgb_projector* p, float* vol, const float* sino,
                   int32_t additive, int32_t bp_kind, void* workspace,
                   int64_t workspace_bytes, void* stream);

/* Forward projection of n volumes stored back to back (item i at
 * vol + i * Nz*Ny*Nx) into n sinograms (sino + i * rows*num_angles*cols), each
 * as tsgb_direct_fp (equal results), in one call. Replaces the per-slice loop
 * over batch and channel dimensions of tomosipo's to_autograd
 * (tomosipo/torch_support.py:49-53). With a workspace of
 * tsgb_fp_batch_workspace_bytes(p, n) bytes, the items run on multi-job
 * launches: one ray launch over as many items as the workspace holds volume
 * copies for (up to 48; the query keeps that within 2 GiB, so projectors
 * whose copies are larger run one item after another); with
 * tsgb_fp_workspace_bytes, one after another on ``stream``. */
int64_t tsgb_fp_batch_workspace_bytes(const tsgb_projector* p, int64_t n);
int tsgb_direct_fp_batch(tsgb_projector* p, const float* vol, float* sino, int64_t n,
                         int32_t additive, void* workspace, int64_t workspace_bytes,
                         void* stream);

/* Backprojection of n sinograms into n volumes, laid out as for
 * tsgb_direct_fp_batch, each as tsgb_direct_bp (equal results). Replaces the
 * per-slice loop of to_autograd's backward pass
 * (tomosipo/torch_support.py:70-74). With a workspace of
 * tsgb_bp_batch_workspace_bytes(p, n, bp_kind) bytes, matched
 * backprojections of the voxel-pair kernel run on multi-job launches (one
 * launch per pass over as many items as the workspace holds weighted
 * sinograms for, up to 48; they fill the GPU where one small volume does not;
 * the query keeps the workspace within 2 GiB); otherwise one item after
 * another. */
int64_t tsgb_bp_batch_workspace_bytes(const tsgb_projector* p, int64_t n, int32_t bp_kind);
int tsgb_direct_bp_batch(tsgb_projector* p, float* vol, const float* sino, int64_t n,
                         int32_t additive, int32_t bp_kind, void* workspace,
                         int64_t workspace_bytes, void* stream);

/* Forward projection of the angles angle_begin .. angle_end - 1 only, into
 * their slices of the full sinogram (other angles untouched). With
 * copies_ready != 0 the padded volume copies a previous call on the same
 * volume left in the workspace are reused. Together with
 * tsgb_copy_sino_angles this lets a caller stream the sinogram to the host
 * while later angles are projected. Results equal tsgb_direct_fp's. Not for
 * projectors with detector supersampling. No counterpart in the reference. */
int tsgb_direct_fp_angles(tsgb_projector* p, const float* vol, float* sino, int32_t additive,
                          int64_t angle_begin, int64_t angle_end, int32_t copies_ready,
                          void* workspace, int64_t workspace_bytes, void* stream);

/* Matched backprojection of the angles angle_begin .. angle_end - 1 of sino
 * (the full sinogram; other angles are not read), vol = ... or vol += ...
 * when ``additive``: a caller can backproject angle chunks as they arrive
 * from the host. The sum over chunks equals tsgb_direct_bp's up to fp32
 * summation order. Not for projectors with detector supersampling. */
int tsgb_direct_bp_angles(tsgb_projector* p, float* vol, const float* sino, int32_t additive,
                          int64_t angle_begin, int64_t angle_end, void* workspace,
                          int64_t workspace_bytes, void* stream);

/* Copy the angles angle_begin .. angle_end - 1 of a rows x num_angles x cols
 * float32 sinogram between host and device (direction from the pointers;
 * asynchronous when the host memory is pinned), one strided 2-D copy. */
int tsgb_copy_sino_angles(void* dst, const void* src, int64_t rows, int64_t num_angles,
                          int64_t cols, int64_t angle_begin, int64_t angle_end, void* stream);

/* Forward projection sino = A(vol) (sino += ... when ``additive``) that allocates
 * no device memory, for callers that cannot call cudaMalloc: code running inside
 * another framework's allocator (a custom-call hook) or a real-time loop with a
 * fixed memory budget. It takes the geometry directly (no projector) plus the
 * caller's input and output, and keeps its scratch -- the padded volume copies
 * and the per-angle parameters -- in fixed static device arrays: at most
 * 16,777,216 floats (64 MiB) of copies (sum of n_d * (n_a + 4) * (n_b + 4) over
 * the axis permutations used; two copies of a 160^3 volume fit) and at most
 * 4096 angles; larger requests fail with TSGB_ERR_INVALID, as do degenerate
 * detectors (the regular projector's checks). The first call on each device
 * resolves the arrays' addresses (make it before any stream capture); the
 * arrays then stay allocated on that device until exit. Calls share the
 * arrays, so calls that overlap on the GPU race: keep them on one stream. The
 * per-angle parameters travel to the device as kernel arguments: a call issues
 * no host-to-device memcpy. No counterpart in the reference (tomosipo / ASTRA). */
int tsgb_direct_fp_noalloc(const tsgb_volume_desc* vol, const tsgb_projection_desc* proj,
                           const float* vol_in, float* sino_out, int32_t additive,
                           void* stream);

/* One job of a batched SIRT solve: x += C * A^T(R * (y - A x)) per iteration.
 * All buffers are device memory on the projector's device: vol, C (volume
 * shaped), sino, R (sinogram shaped), residual (2 * (rows + 4) * angles * cols
 * floats, zeroed by the caller once: the backprojector's row-pair layout with
 * two padding rows above and below the detector), fp_workspace
 * (tsgb_fp_workspace_bytes). Any geometry without detector supersampling:
 * angles whose det_v runs along z (circular and helical scans) take the
 * separable backprojector with the update fused into its epilogue, others
 * (tilted detectors) the general one followed by an element-wise update. */
typedef struct {
  tsgb_projector* projector;
  float* vol;
  const float* sino;
  const float* R;
  const float* C;
  float* residual;
  float* fp_workspace;
} tsgb_sirt_job;

typedef struct tsgb_sirt_batch tsgb_sirt_batch;

/* Build a batch: orders the jobs largest first and creates its streams (at
 * most 8) and events on the current device. No counterpart in the reference,
 * whose SIRT is a Python loop per job (README.md:150-163); results are bitwise
 * equal to that loop's. */
int tsgb_sirt_batch_create(const tsgb_sirt_job* jobs, int32_t n_jobs, tsgb_sirt_batch** out);

/* Run ``iterations`` SIRT iterations of every job. Per job and iteration: its
 * padded volume copies, the forward projection writing the residual and the
 * backprojection applying the update, on the batch's streams, forked from and
 * joined back into ``stream`` (jobs never wait for each other). Allocates
 * nothing; capturable in a CUDA graph (the fork and join become its
 * branches). */
int tsgb_sirt_batch_iterate(tsgb_sirt_batch* b, int32_t iterations, void* stream);

/* As tsgb_sirt_batch_iterate, with iterations[i] iterations of job i (the
 * order of tsgb_sirt_batch_create's ``jobs``; 0 leaves a job as it is), so a
 * scheduler can advance jobs unevenly from one batch. */
int tsgb_sirt_batch_iterate_jobs(tsgb_sirt_batch* b, const int32_t* iterations, void* stream);

/* Free a batch's tables (not the jobs' buffers). */
int tsgb_sirt_batch_destroy(tsgb_sirt_batch* b);

/* Launch schedule of a projector's forward projection (the order of its
 * independent tiles; a tile is 32 detector rows x 8 columns of one pair of
 * adjacent angles). The detector is cut into patches of fp_patch_rows x
 * fp_patch_cols tiles and the angles into groups of fp_group_pairs pairs;
 * a group's tiles over one patch run together, so the volume slab their rays
 * cross is read from HBM once and reused from L2 across the group's angles.
 * Any values >= 1 give bit-identical results. bp_kernel and bp_shape pick the
 * matched backprojector and its warp shape; they change only the order of
 * fp32 sums. bp_general picks the kernel of angles outside that backprojector. Defaults are set at creation; the Python autotuner times
 * candidates and sets the fastest. Used by tsgb_direct_fp / tsgb_direct_bp and
 * by the batched SIRT passes. No counterpart in the reference (ASTRA's launch
 * shapes are fixed). */
typedef struct {
  int32_t fp_patch_rows;  /* tiles of 32 detector rows per patch (>= 1) */
  int32_t fp_patch_cols;  /* tiles of 8 detector columns per patch (>= 1) */
  int32_t fp_group_pairs; /* pairs of adjacent angles per group (>= 1) */
  int32_t fp_pair_layout; /* 1: volume copies hold neighbour pairs (two 8-byte
                             loads per sample), 0: single voxels (four 4-byte) */
  int32_t bp_kernel;      /* matched backprojection of det_v-along-z angles:
                             1: z-lane warps over a column-major weighted
                             sinogram, 0: voxel-pair threads over a row-major one */
  int32_t bp_shape;       /* z-lane warp shape (voxels along the in-plane axis x
                             voxels along z per lane x warps per block):
                             0: 4x8x4, 1: 4x8x8, 2: 4x16x8, 3: 4x16x16,
                             4: 3x16x8, 5: 4x4x4, 6: 4x2x4 */
  int32_t bp_general;     /* matched backprojection of the other angles (tilted
                             detectors): 0: blocks over voxel boxes that stage
                             each angle's detector region in shared memory,
                             1: one thread per voxel; both give the same sums */
  int32_t reserved;       /* must be 0 */
} tsgb_tuning;

int tsgb_projector_get_tuning(const tsgb_projector* p, tsgb_tuning* out);
int tsgb_projector_set_tuning(tsgb_projector* p, const tsgb_tuning* t);

/* FDK backprojection (the backprojection step of tomosipo's fdk,
 * tomosipo/astra.py:374-406, which calls ASTRA's accumulate_FDK): for any
 * cone beam (circular, helical, rotated or tilted-detector scans),
 *   vol (+)= sum_t angle_weights[t] * q_t(u_t(x), v_t(x)) / w_t(x)^2
 * where q is the already weighted and ramp-filtered sinogram (layout as any
 * sinogram), read with bilinear interpolation and zero outside the detector,
 * and w_t(x) is the voxel's depth along the detector normal divided by the
 * volume anchor's (the centre of voxel (nz/2, ny/2, nx/2)). angle_weights is a
 * device array of num_angles floats. Workspace: tsgb_bp_workspace_bytes(p,
 * TSGB_BP_BILINEAR). The weighting and filtering steps are the caller's
 * (tomosipo_gb300/fdk.py). */
int tsgb_fdk_backproject(tsgb_projector* p, float* vol, const float* filtered,
                         const float* angle_weights, int32_t additive, void* workspace,
                         int64_t workspace_bytes, void* stream);

/* Shapes the projector expects: vol (z, y, x) and sino (rows, angles, cols). */
int tsgb_projector_shapes(const tsgb_projector* p, int64_t vol_shape[3],
                          int64_t sino_shape[3]);

/* Plan statistics, written to out[0..n-1] (n <= 8):
 *   [0] padded volume copies the forward projector builds (axis permutations)
 *   [1] angles backprojected by the separable (det_v along z) gather kernel
 *   [2] angles backprojected by the general gather kernel
 *   [3] kernel launches per tsgb_direct_fp call
 *   [4] kernel launches per matched tsgb_direct_bp call
 *   [5] kernel launches per bilinear tsgb_direct_bp call
 *   [6] forward workspace bytes, [7] matched backprojection workspace bytes
 * No counterpart in ASTRA's projector; used for measurement and tests. */
int tsgb_projector_stats(const tsgb_projector* p, int64_t* out, int32_t n);

/* Message for the calling thread's most recent error ("" if none). */
const char* tsgb_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* TOMOSIPO_GB300_H */
