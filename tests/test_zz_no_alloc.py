"""The allocation-free forward projection, tsgb_direct_fp_noalloc.

It serves callers that cannot call cudaMalloc (code inside another framework's
allocator, real-time loops with a fixed memory budget): they hand over only the
geometry, their input volume and their output sinogram, and the projector keeps
its scratch in fixed static device arrays. This file is collected last so that a
run stopping at the first failure has run every other test first; it also passes
alone in a fresh process.

The check: two calls in a row through the C ABI agree with the projector's
regular entry point (ts.operator -> tsgb_direct_fp) within the parity tolerance.
"""
import ctypes

import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300 import _native
from tomosipo_gb300.projector import projection_vectors
from tests.helpers import TOL_ORACLE, ellipsoid_phantom, noise_cube_phantom, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _descriptors(vg, pg):
    v = _native.VolumeDesc()
    v.shape[:] = list(vg.shape)
    v.pos[:] = [float(x) for x in vg.pos[0]]
    v.size[:] = [float(x) for x in vg.size]
    kind, rows, cols, vec = projection_vectors(pg)
    p = _native.ProjectionDesc()
    p.kind = kind
    p.det_shape[:] = [rows, cols]
    p.num_angles = vec.shape[0]
    p.vectors = vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return v, p, vec


@pytest.mark.parametrize(
    "geometry",
    [
        lambda: (ts.volume(shape=64, size=1),
                 ts.cone(angles=48, shape=(64, 96), size=np.sqrt(2), cone_angle=0.5)),
        lambda: (ts.volume(shape=(40, 48, 56), size=(0.9, 1.0, 1.1)),
                 ts.parallel(angles=30, shape=(44, 70), size=(1.2, 1.8))),
    ],
)
def test_noalloc_fp_matches_regular_entry_point(native_lib, geometry):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda", 0)
    vg, pg = geometry()
    A = ts.operator(vg, pg)
    v, p, _keep = _descriptors(vg, pg)
    stream = torch.cuda.current_stream(dev).cuda_stream
    inputs = [noise_cube_phantom(vg.shape, seed=21), ellipsoid_phantom(vg.shape, n=5, seed=22)]
    for x_np in inputs:  # two calls in a row, different inputs
        x = torch.from_numpy(x_np).to(dev)
        expected = A(x)
        out = torch.full(A.range_shape, float("nan"), device=dev)
        rc = native_lib.tsgb_direct_fp_noalloc(ctypes.byref(v), ctypes.byref(p), x.data_ptr(),
                                              out.data_ptr(), 0, stream)
        assert rc == 0, native_lib.tsgb_last_error().decode()
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        assert rel_l2(out.cpu().numpy(), expected.cpu().numpy()) <= TOL_ORACLE


def test_noalloc_fp_rejects_oversized_requests(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vg = ts.volume(shape=(300, 300, 300), size=1)
    pg = ts.cone(angles=4, shape=(300, 300), size=np.sqrt(2), cone_angle=0.5)
    v, p, _keep = _descriptors(vg, pg)
    x = torch.zeros(1, device="cuda")
    out = torch.zeros(1, device="cuda")
    rc = native_lib.tsgb_direct_fp_noalloc(ctypes.byref(v), ctypes.byref(p), x.data_ptr(),
                                          out.data_ptr(), 0, None)
    assert rc == -1
    assert "at most" in native_lib.tsgb_last_error().decode()
