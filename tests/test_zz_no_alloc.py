"""The allocation-free forward projection, tsgb_direct_fp_noalloc.

It serves callers that cannot call cudaMalloc (code inside another framework's
allocator, real-time loops with a fixed memory budget): they hand over only the
geometry, their input volume and their output sinogram, and the projector keeps
its scratch in fixed static device arrays. This file is collected last so that a
run stopping at the first failure has run every other test first; it also passes
alone in a fresh process.

The checks: two calls in a row through the C ABI agree with the projector's
regular entry point (ts.operator -> tsgb_direct_fp) and with the FP64 oracle
within the parity tolerance, for circular, helical and rotated vector
geometries; the additive form adds; a small request after a large one sees no
stale scratch; the size limits and degenerate detectors are rejected; and
calls after the first change no device memory.
"""
import ctypes

import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300 import _native
from tomosipo_gb300.projector import projection_vectors
from oracle import oracle as orc
from tests.helpers import (TOL_ORACLE, ellipsoid_phantom, helical_cone_vec, noise_cube_phantom,
                           rel_l2)

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


GEOMETRIES = {
    "cone": lambda: (ts.volume(shape=64, size=1),
                     ts.cone(angles=48, shape=(64, 96), size=np.sqrt(2), cone_angle=0.5)),
    "parallel_aniso": lambda: (ts.volume(shape=(40, 48, 56), size=(0.9, 1.0, 1.1)),
                               ts.parallel(angles=30, shape=(44, 70), size=(1.2, 1.8))),
    # helical source/detector path with per-angle jitter (det_v along z)
    "cone_vec_helical": lambda: (ts.volume(shape=32, size=1),
                                 helical_cone_vec(40, (24, 40), (1.0, 1.6), 2.5, 1.0, pitch=0.3,
                                                  turns=1.5, jitter=0.5, voxel=1 / 32)),
    # a rotated scan: other axis permutations of the dominant / in-plane axes
    "cone_vec_rotated": lambda: (
        ts.volume(shape=(24, 28, 32), size=(0.8, 0.9, 1.0)),
        ts.rotate(pos=0, axis=(1.0, 0.3, -0.2), angles=0.9)
        * ts.cone(angles=20, shape=(36, 44), size=1.6, src_orig_dist=2.5, src_det_dist=3.5).to_vec()),
}


def _call(lib, v, p, x, out, additive, stream):
    rc = lib.tsgb_direct_fp_noalloc(ctypes.byref(v), ctypes.byref(p), x.data_ptr(), out.data_ptr(),
                                    additive, stream)
    assert rc == 0, lib.tsgb_last_error().decode()


@pytest.fixture(scope="module")
def dev(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.mark.parametrize("name", sorted(GEOMETRIES))
def test_noalloc_fp_matches_regular_entry_point(native_lib, dev, name):
    vg, pg = GEOMETRIES[name]()
    A = ts.operator(vg, pg)
    v, p, _keep = _descriptors(vg, pg)
    stream = torch.cuda.current_stream(dev).cuda_stream
    inputs = [noise_cube_phantom(vg.shape, seed=21), ellipsoid_phantom(vg.shape, n=5, seed=22)]
    for x_np in inputs:  # two calls in a row, different inputs
        x = torch.from_numpy(x_np).to(dev)
        expected = A(x)
        out = torch.full(A.range_shape, float("nan"), device=dev)
        _call(native_lib, v, p, x, out, 0, stream)
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        got = out.cpu().numpy()
        assert rel_l2(got, expected.cpu().numpy()) <= TOL_ORACLE
        # and against the FP64 oracle itself, not only the other GPU path
        assert rel_l2(got, orc.fp(vg, pg, x_np)) <= TOL_ORACLE


def test_noalloc_additive_adds(native_lib, dev):
    """additive=1 adds onto the output: a set call then an additive call give 2 A(x)."""
    vg, pg = GEOMETRIES["cone_vec_helical"]()
    v, p, _keep = _descriptors(vg, pg)
    x_np = noise_cube_phantom(vg.shape, seed=23)
    x = torch.from_numpy(x_np).to(dev)
    out = torch.full(ts.operator(vg, pg).range_shape, float("nan"), device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _call(native_lib, v, p, x, out, 0, stream)
    _call(native_lib, v, p, x, out, 1, stream)
    torch.cuda.synchronize()
    assert rel_l2(out.cpu().numpy(), 2 * orc.fp(vg, pg, x_np)) <= TOL_ORACLE


def test_noalloc_small_after_large_sees_no_stale_scratch(native_lib, dev):
    """A large request fills more of the shared scratch (and more parameter
    slots) than the small one after it; the small result must equal the
    regular entry point's, as if it ran first."""
    stream = torch.cuda.current_stream(dev).cuda_stream
    big_vg = ts.volume(shape=150, size=1)
    big_pg = ts.cone(angles=300, shape=(150, 220), size=np.sqrt(2), cone_angle=0.5)
    vb, pb, _kb = _descriptors(big_vg, big_pg)
    xb = torch.from_numpy(ellipsoid_phantom(big_vg.shape, n=6, seed=24)).to(dev)
    ob = torch.empty(ts.operator(big_vg, big_pg).range_shape, device=dev)
    _call(native_lib, vb, pb, xb, ob, 0, stream)
    vg, pg = GEOMETRIES["cone_vec_rotated"]()
    A = ts.operator(vg, pg)
    v, p, _keep = _descriptors(vg, pg)
    x = torch.from_numpy(noise_cube_phantom(vg.shape, seed=25)).to(dev)
    out = torch.full(A.range_shape, float("nan"), device=dev)
    _call(native_lib, v, p, x, out, 0, stream)
    torch.cuda.synchronize()
    assert rel_l2(out.cpu().numpy(), A(x).cpu().numpy()) <= TOL_ORACLE


def test_noalloc_calls_change_no_device_memory(native_lib, dev):
    """After the first call on the device (which may load the module and its
    static arrays), further calls leave the device's free memory unchanged."""
    vg, pg = GEOMETRIES["cone"]()
    v, p, _keep = _descriptors(vg, pg)
    x = torch.from_numpy(noise_cube_phantom(vg.shape, seed=26)).to(dev)
    out = torch.empty(ts.operator(vg, pg).range_shape, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _call(native_lib, v, p, x, out, 0, stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    for additive in (0, 1, 0, 1):
        _call(native_lib, v, p, x, out, additive, stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free0


def test_noalloc_angle_limit(native_lib, dev):
    """4096 angles are accepted, 4097 rejected with a message."""
    vg = ts.volume(shape=8, size=1)
    x = torch.from_numpy(noise_cube_phantom(vg.shape, seed=27)).to(dev)
    for nang, ok in ((4096, True), (4097, False)):
        pg = ts.parallel(angles=nang, shape=(8, 12), size=(1, 1.5))
        v, p, _keep = _descriptors(vg, pg)
        out = torch.empty((8, nang, 12), device=dev)
        rc = native_lib.tsgb_direct_fp_noalloc(ctypes.byref(v), ctypes.byref(p), x.data_ptr(),
                                              out.data_ptr(), 0, None)
        if ok:
            assert rc == 0, native_lib.tsgb_last_error().decode()
            torch.cuda.synchronize()
            assert rel_l2(out.cpu().numpy(), orc.fp(vg, pg, x.cpu().numpy())) <= TOL_ORACLE
        else:
            assert rc == -1
            assert "4096" in native_lib.tsgb_last_error().decode()


def test_noalloc_rejects_degenerate_detectors(native_lib, dev):
    """A zero det_u, or det_u parallel to det_v, is TSGB_ERR_INVALID, as the
    regular projector's planner rejects it."""
    vg = ts.volume(shape=8, size=1)
    pg = ts.cone(angles=4, shape=(8, 12), size=np.sqrt(2), cone_angle=0.5)
    x = torch.zeros(vg.shape, device=dev)
    out = torch.zeros((8, 4, 12), device=dev)
    for bad in ("zero_u", "parallel"):
        v, p, vec = _descriptors(vg, pg)
        vec[2, 9:12] = 0.0 if bad == "zero_u" else 2.0 * vec[2, 6:9]
        rc = native_lib.tsgb_direct_fp_noalloc(ctypes.byref(v), ctypes.byref(p), x.data_ptr(),
                                              out.data_ptr(), 0, None)
        assert rc == -1
        assert "degenerate detector" in native_lib.tsgb_last_error().decode()


def test_noalloc_fp_rejects_oversized_requests(native_lib, dev):
    vg = ts.volume(shape=(300, 300, 300), size=1)
    pg = ts.cone(angles=4, shape=(300, 300), size=np.sqrt(2), cone_angle=0.5)
    v, p, _keep = _descriptors(vg, pg)
    x = torch.zeros(1, device="cuda")
    out = torch.zeros(1, device="cuda")
    rc = native_lib.tsgb_direct_fp_noalloc(ctypes.byref(v), ctypes.byref(p), x.data_ptr(),
                                          out.data_ptr(), 0, None)
    assert rc == -1
    assert "at most" in native_lib.tsgb_last_error().decode()
