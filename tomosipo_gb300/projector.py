"""GB300 link layer: replaces tomosipo's ``tomosipo/astra.py`` (lines 80-217).

``create_projector`` plays the role of ``create_astra_projector``
(``astra.py:80-98``) and ``direct_fp`` / ``direct_bp`` the role of the
functions that call ``astra.experimental.direct_FPBP3D`` (``astra.py:104-217``),
with the same argument meaning and the same ``ValueError`` on device mismatch.
Work runs on the current CUDA stream of the data's device, asynchronously.
Host (NumPy / CPU tensor) data are staged through the current CUDA device;
without a CUDA device every projection raises ``RuntimeError``.
"""
import ctypes

import numpy as np
import torch

from . import _native
from .geometry import VolumeGeometry, is_volume
from .links.base import are_compatible

BP_KINDS = {"matched": _native.TSGB_BP_MATCHED, "bilinear": _native.TSGB_BP_BILINEAR}


def projection_vectors(pg):
    """(kind, rows, cols, vectors[num_angles, 12]) of a projection geometry.

    Row layout: [src_pos or ray_dir, det_pos, det_v, det_u], each (z, y, x).
    Anything but a parallel or cone geometry (vector or not) is a TypeError:
    a volume, or a detector alone, defines no rays.
    """
    if not (getattr(pg, "is_parallel", False) or getattr(pg, "is_cone", False)):
        raise TypeError(
            "Expected a parallel or cone projection geometry (ts.parallel, ts.parallel_vec, "
            f"ts.cone, ts.cone_vec). Got {type(pg).__name__}."
        )
    v = pg.to_vec()
    first = v.src_pos if pg.is_cone else v.ray_dir
    vec = np.concatenate([first, v.det_pos, v.det_v, v.det_u], axis=1)
    kind = _native.TSGB_CONE if pg.is_cone else _native.TSGB_PARALLEL
    rows, cols = v.det_shape
    return kind, rows, cols, np.ascontiguousarray(vec, dtype=np.float64)


class Projector:
    """Geometry of one (volume, projection) pair plus its native handles.

    Native projectors are created lazily, one per CUDA device, and freed with
    this object (ASTRA projector ids in the reference are never freed).
    """

    def __init__(self, vg, pg, voxel_supersampling=1, detector_supersampling=1):
        if not isinstance(vg, VolumeGeometry):
            raise TypeError(f"Expected an axis-aligned VolumeGeometry. Got {type(vg)}.")
        self.vg = vg
        self.pg = pg
        self.voxel_supersampling = int(voxel_supersampling)
        self.detector_supersampling = int(detector_supersampling)
        kind, rows, cols, vec = projection_vectors(pg)
        self._vectors = vec  # kept alive: the descriptor points into it
        self.vol_desc = _native.VolumeDesc()
        self.vol_desc.shape[:] = list(vg.shape)
        self.vol_desc.pos[:] = [float(x) for x in vg.pos[0]]
        self.vol_desc.size[:] = [float(x) for x in vg.size]
        self.proj_desc = _native.ProjectionDesc()
        self.proj_desc.kind = kind
        self.proj_desc.det_shape[:] = [rows, cols]
        self.proj_desc.num_angles = vec.shape[0]
        self.proj_desc.vectors = vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self.vol_shape = tuple(vg.shape)
        self.sino_shape = (rows, vec.shape[0], cols)
        self._handles = {}

    def handle(self, device_index):
        h = self._handles.get(device_index)
        if h is None:
            lib = _native.load()
            out = ctypes.c_void_p()
            with torch.cuda.device(device_index):
                rc = lib.tsgb_projector_create(
                    ctypes.byref(self.vol_desc),
                    ctypes.byref(self.proj_desc),
                    self.voxel_supersampling,
                    self.detector_supersampling,
                    ctypes.byref(out),
                )
            _native.check(rc, "tsgb_projector_create")
            h = out.value
            self._handles[device_index] = h
        return h

    def workspace_bytes(self, device_index, forward, bp_kind="matched"):
        lib = _native.load()
        h = self.handle(device_index)
        if forward:
            return int(lib.tsgb_fp_workspace_bytes(h))
        return int(lib.tsgb_bp_workspace_bytes(h, BP_KINDS[bp_kind]))

    def stats(self, device_index):
        """Plan statistics of the native projector (see tsgb_projector_stats)."""
        lib = _native.load()
        out = (ctypes.c_int64 * 8)()
        _native.check(lib.tsgb_projector_stats(self.handle(device_index), out, 8),
                      "tsgb_projector_stats")
        keys = ["layouts", "separable_bp_angles", "general_bp_angles", "fp_launches",
                "bp_matched_launches", "bp_bilinear_launches", "fp_workspace_bytes",
                "bp_workspace_bytes"]
        return dict(zip(keys, [int(v) for v in out]))

    TUNING_KEYS = ("fp_patch_rows", "fp_patch_cols", "fp_group_pairs", "fp_pair_layout",
                   "bp_kernel", "bp_shape", "bp_general")

    def get_tuning(self, device_index=None):
        """Launch schedule of the forward projector (see tsgb_tuning)."""
        lib = _native.load()
        t = _native.Tuning()
        _native.check(lib.tsgb_projector_get_tuning(self.handle(_device_index(device_index)),
                                                    ctypes.byref(t)), "tsgb_projector_get_tuning")
        return {k: int(getattr(t, k)) for k in self.TUNING_KEYS}

    def set_tuning(self, device_index=None, **values):
        """Change schedule values (keys of ``get_tuning``); results stay bit-identical."""
        unknown = set(values) - set(self.TUNING_KEYS)
        if unknown:
            raise ValueError(f"unknown tuning keys {sorted(unknown)}")
        idx = _device_index(device_index)
        cur = self.get_tuning(idx)
        cur.update({k: int(v) for k, v in values.items()})
        t = _native.Tuning(**cur)
        _native.check(_native.load().tsgb_projector_set_tuning(self.handle(idx), ctypes.byref(t)),
                      "tsgb_projector_set_tuning")

    def __del__(self):
        handles, self._handles = getattr(self, "_handles", {}), {}
        if handles and _native._lib is not None:
            for h in handles.values():
                try:
                    _native._lib.tsgb_projector_destroy(h)
                except Exception:  # a finalizer: at interpreter exit CUDA may be torn down
                    pass


def _device_index(device_index):
    if device_index is None:
        return torch.cuda.current_device()
    return int(device_index)


def create_projector(volume_geometry, projection_geometry, *, voxel_supersampling=1,
                     detector_supersampling=1):
    """Projector for an axis-aligned volume and any projection geometry."""
    if not is_volume(volume_geometry) or not isinstance(volume_geometry, VolumeGeometry):
        raise TypeError("create_projector expects an axis-aligned VolumeGeometry")
    if voxel_supersampling < 1 or detector_supersampling < 1:
        raise ValueError("supersampling factors must be >= 1")
    return Projector(volume_geometry, projection_geometry, voxel_supersampling,
                     detector_supersampling)


# tomosipo name for the same function (tomosipo/astra.py:80)
create_astra_projector = create_projector


def _cuda_device_for_host_data():
    if not torch.cuda.is_available():
        raise RuntimeError(
            "tomosipo_gb300 projects on a CUDA GPU only; no CUDA device is available "
            "(there is no CPU fallback)."
        )
    return torch.device("cuda", torch.cuda.current_device())


def _as_device_tensor(arr, device, copy_in):
    """Device tensor view of a link's data; returns (tensor, needs_copy_back)."""
    if isinstance(arr, torch.Tensor) and arr.is_cuda:
        return arr, False
    t = torch.from_numpy(arr) if isinstance(arr, np.ndarray) else arr
    if copy_in:
        return t.to(device, non_blocking=False), True
    return torch.empty(t.shape, dtype=torch.float32, device=device), True


# Host data: stream the sinogram between host and device in angle chunks,
# overlapped with the projection of the other chunks, when it is at least this
# large (tsgb_direct_fp_angles / tsgb_direct_bp_angles / tsgb_copy_sino_angles).
PIPELINE_MIN_BYTES = 256 << 20
PIPELINE_MIN_ANGLES = 16
# Chunk sizes grow by these factors from the chunk whose transfer is exposed.
# At full copy rates a projection takes 15-20x longer per angle than its
# transfer at 512^3 (127-141 us against 7.5 us). Every backprojection chunk
# rereads and rewrites the volume, so its chunks grow by 8: few chunks. A
# forward chunk costs nothing extra (the volume copies are built once), and
# downloads into host memory have measured as slow as 24 GB/s on a shared
# host (193 GB/s otherwise), about twice the rate the forward projection
# produces sinogram; chunks growing by 2 keep each download behind the
# projection of the chunks after it even then.
PIPELINE_GROWTH_BP = 8
PIPELINE_GROWTH_FP = 2
_copy_streams = {}


def _chunk_bounds(nang, forward):
    """Angle-chunk bounds for a pipelined projection.

    The backprojection's first chunk waits for its upload and the forward
    projection's last chunk for its download, so that chunk is small (1/32
    of the angles) and the others grow geometrically away from it (by
    PIPELINE_GROWTH_BP or PIPELINE_GROWTH_FP); the farthest chunk also takes
    what is left. Forward chunks run from the farthest to the exposed one.
    """
    growth = PIPELINE_GROWTH_FP if forward else PIPELINE_GROWTH_BP
    sizes, left, size = [], nang, max(1, nang // 32)
    while left > 0:
        sizes.append(min(size, left))
        left -= sizes[-1]
        size *= growth
    if len(sizes) > 1 and sizes[-1] < sizes[-2]:
        rest = sizes.pop()  # a remainder smaller than its neighbour joins it
        sizes[-1] += rest
    if forward:
        sizes.reverse()
    return np.concatenate([[0], np.cumsum(sizes)]).astype(int)


def _host_ptr(arr):
    return arr.ctypes.data if isinstance(arr, np.ndarray) else arr.data_ptr()


class TransferTimeline:
    """CUDA-event spans of host-data projections, for measurement.

    While installed with ``record_transfers(timeline)``, every pipelined
    host-to-host projection records labelled spans on the stream each step
    runs on: ``vol_h2d``, ``fp`` chunks and ``sino_d2h`` chunks in the forward
    leg; ``sino_h2d`` chunks, ``bp`` chunks and ``vol_d2h`` in the backward
    leg; and the whole leg (``fp_leg`` / ``bp_leg``). ``summary()`` (after the
    device is synchronised) sums each label's milliseconds.
    """

    def __init__(self):
        self.spans = []

    def begin(self, label, stream):
        e = torch.cuda.Event(enable_timing=True)
        e.record(stream)
        return (label, e)

    def end(self, token, stream):
        label, e0 = token
        e1 = torch.cuda.Event(enable_timing=True)
        e1.record(stream)
        self.spans.append((label, e0, e1))

    def summary(self):
        out = {}
        for label, e0, e1 in self.spans:
            out[label] = out.get(label, 0.0) + e0.elapsed_time(e1)
        return out


_timeline = None


class record_transfers:
    """Context manager installing a TransferTimeline for host-data projections."""

    def __init__(self, timeline):
        self.timeline = timeline

    def __enter__(self):
        global _timeline
        self._prev, _timeline = _timeline, self.timeline
        return self.timeline

    def __exit__(self, *exc):
        global _timeline
        _timeline = self._prev
        return False


def _begin(label, stream):
    return _timeline.begin(label, stream) if _timeline is not None else None


def _end(token, stream):
    if token is not None and _timeline is not None:
        _timeline.end(token, stream)


def _pipelined(projector, forward, additive, bp_kind, src, dst):
    """Both buffers on the host and large enough to hide their transfers."""
    rows, nang, cols = projector.sino_shape
    return (projector.detector_supersampling == 1 and (forward or bp_kind == "matched")
            and 4 * rows * nang * cols >= PIPELINE_MIN_BYTES and nang >= PIPELINE_MIN_ANGLES)


def _project_pipelined(projector, forward, additive, src, dst, device):
    """Host-to-host projection with the sinogram streamed in angle chunks.

    Forward: the volume goes in, then chunk c is projected while chunk c - 1
    is copied out. Backward (matched): chunk c is copied in while chunk c - 1
    is backprojected into the volume, which then comes out. Results equal the
    one-call path (the backprojection up to fp32 summation order).
    """
    lib = _native.load()
    rows, nang, cols = projector.sino_shape
    bounds = _chunk_bounds(nang, forward)
    chunks = len(bounds) - 1
    with torch.cuda.device(device):
        h = projector.handle(device.index)
        comp = torch.cuda.current_stream(device)
        copy = _copy_streams.setdefault(device.index, torch.cuda.Stream(device))
        nbytes = projector.workspace_bytes(device.index, forward, "matched")
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=device)
        start = torch.cuda.Event()
        if forward:
            leg = _begin("fp_leg", comp)
            t = _begin("vol_h2d", comp)
            d_vol, _ = _as_device_tensor(src, device, copy_in=True)
            _end(t, comp)
            d_sino, _ = _as_device_tensor(dst, device, copy_in=additive)
            start.record(comp)
            copy.wait_event(start)
            for c in range(chunks):
                a0, a1 = int(bounds[c]), int(bounds[c + 1])
                t = _begin("fp", comp)
                _native.check(lib.tsgb_direct_fp_angles(h, d_vol.data_ptr(), d_sino.data_ptr(),
                                                        int(bool(additive)), a0, a1, int(c > 0),
                                                        ws.data_ptr(), nbytes, comp.cuda_stream),
                              "tsgb_direct_fp_angles")
                _end(t, comp)
                done = torch.cuda.Event()
                done.record(comp)
                copy.wait_event(done)
                t = _begin("sino_d2h", copy)
                _native.check(lib.tsgb_copy_sino_angles(_host_ptr(dst), d_sino.data_ptr(), rows,
                                                        nang, cols, a0, a1, copy.cuda_stream),
                              "tsgb_copy_sino_angles")
                _end(t, copy)
            finished = torch.cuda.Event()
            finished.record(copy)
            comp.wait_event(finished)
            _end(leg, comp)
            copy.synchronize()
        else:
            leg = _begin("bp_leg", comp)
            d_sino = torch.empty((rows, nang, cols), dtype=torch.float32, device=device)
            d_vol, _ = _as_device_tensor(dst, device, copy_in=additive)
            start.record(comp)
            copy.wait_event(start)
            for c in range(chunks):
                a0, a1 = int(bounds[c]), int(bounds[c + 1])
                t = _begin("sino_h2d", copy)
                _native.check(lib.tsgb_copy_sino_angles(d_sino.data_ptr(), _host_ptr(src), rows,
                                                        nang, cols, a0, a1, copy.cuda_stream),
                              "tsgb_copy_sino_angles")
                _end(t, copy)
                arrived = torch.cuda.Event()
                arrived.record(copy)
                comp.wait_event(arrived)
                t = _begin("bp", comp)
                _native.check(lib.tsgb_direct_bp_angles(h, d_vol.data_ptr(), d_sino.data_ptr(),
                                                        int(bool(additive) or c > 0), a0, a1,
                                                        ws.data_ptr(), nbytes, comp.cuda_stream),
                              "tsgb_direct_bp_angles")
                _end(t, comp)
            target = torch.from_numpy(dst) if isinstance(dst, np.ndarray) else dst
            t = _begin("vol_d2h", comp)
            target.copy_(d_vol)
            _end(t, comp)
            _end(leg, comp)


def direct_project(projector, vol_link, proj_link, forward=None, additive=False,
                   bp_kind="matched"):
    """Forward (``forward=True``) or back project between two links."""
    if forward is None:
        raise ValueError("project must be given a forward argument (True/False).")
    if bp_kind not in BP_KINDS:
        raise ValueError(f"bp_kind must be one of {sorted(BP_KINDS)}. Got {bp_kind!r}.")
    if not are_compatible(vol_link, proj_link):
        raise ValueError(
            "Cannot perform projection on volume and projection data, because they are "
            "not compatible. Usually, this indicates that the data are located on "
            "different computing devices. "
        )
    if tuple(vol_link.shape) != projector.vol_shape or tuple(proj_link.shape) != projector.sino_shape:
        raise ValueError(
            f"Expected volume {projector.vol_shape} and sinogram {projector.sino_shape}. "
            f"Got {tuple(vol_link.shape)} and {tuple(proj_link.shape)}."
        )
    # device-array links (CuPy and the like) project through a torch view
    vol = getattr(vol_link, "torch_view", None)
    vol = vol_link.data if vol is None else vol
    sino = getattr(proj_link, "torch_view", None)
    sino = proj_link.data if sino is None else sino
    on_gpu = isinstance(vol, torch.Tensor) and vol.is_cuda
    device = vol.device if on_gpu else _cuda_device_for_host_data()
    src, dst = (vol, sino) if forward else (sino, vol)
    if not on_gpu and _pipelined(projector, forward, additive, bp_kind, src, dst):
        return _project_pipelined(projector, forward, additive, src, dst, device)
    d_src, _ = _as_device_tensor(src, device, copy_in=True)
    d_dst, copy_back = _as_device_tensor(dst, device, copy_in=additive)
    lib = _native.load()
    with torch.cuda.device(device):
        h = projector.handle(device.index)
        stream = torch.cuda.current_stream(device).cuda_stream
        nbytes = projector.workspace_bytes(device.index, forward, bp_kind)
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=device)
        if forward:
            rc = lib.tsgb_direct_fp(h, d_src.data_ptr(), d_dst.data_ptr(), int(bool(additive)),
                                    ws.data_ptr(), nbytes, stream)
        else:
            rc = lib.tsgb_direct_bp(h, d_dst.data_ptr(), d_src.data_ptr(), int(bool(additive)),
                                    BP_KINDS[bp_kind], ws.data_ptr(), nbytes, stream)
        _native.check(rc, "tsgb_direct_fp" if forward else "tsgb_direct_bp")
    if copy_back:
        # Straight device -> host copy into the caller's buffer (a DMA when it is pinned).
        target = torch.from_numpy(dst) if isinstance(dst, np.ndarray) else dst
        target.copy_(d_dst)


def direct_project_batch(projector, vol, sino, forward, additive=False, bp_kind="matched"):
    """Project item i of ``vol`` (n, z, y, x) to/from item i of ``sino``
    (n, rows, angles, cols) for every i in one C-ABI call: CUDA float32
    C-contiguous tensors on one device (no coercion; callers check)."""
    if bp_kind not in BP_KINDS:
        raise ValueError(f"bp_kind must be one of {sorted(BP_KINDS)}. Got {bp_kind!r}.")
    n = vol.shape[0]
    if (tuple(vol.shape[1:]) != projector.vol_shape or tuple(sino.shape[1:]) != projector.sino_shape
            or sino.shape[0] != n):
        raise ValueError(
            f"Expected volumes (n, {projector.vol_shape}) and sinograms (n, {projector.sino_shape}). "
            f"Got {tuple(vol.shape)} and {tuple(sino.shape)}.")
    if vol.device != sino.device or not vol.is_cuda:
        raise ValueError("batched projection needs both tensors on the same CUDA device")
    device = vol.device
    lib = _native.load()
    with torch.cuda.device(device):
        h = projector.handle(device.index)
        stream = torch.cuda.current_stream(device).cuda_stream
        # per-item volume copies / weighted sinograms let the items share launches
        if forward:
            nbytes = int(lib.tsgb_fp_batch_workspace_bytes(h, n))
        else:
            nbytes = int(lib.tsgb_bp_batch_workspace_bytes(h, n, BP_KINDS[bp_kind]))
        if nbytes < 0:
            _native.check(nbytes, "batch workspace query")
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=device)
        if forward:
            rc = lib.tsgb_direct_fp_batch(h, vol.data_ptr(), sino.data_ptr(), n, int(bool(additive)),
                                          ws.data_ptr(), nbytes, stream)
        else:
            rc = lib.tsgb_direct_bp_batch(h, vol.data_ptr(), sino.data_ptr(), n, int(bool(additive)),
                                          BP_KINDS[bp_kind], ws.data_ptr(), nbytes, stream)
        _native.check(rc, "tsgb_direct_fp_batch" if forward else "tsgb_direct_bp_batch")


def direct_fp(projector, vol_data, proj_data, additive=False):
    return direct_project(projector, vol_data, proj_data, forward=True, additive=additive)


def direct_bp(projector, vol_data, proj_data, additive=False, bp_kind="matched"):
    return direct_project(projector, vol_data, proj_data, forward=False, additive=additive,
                          bp_kind=bp_kind)
