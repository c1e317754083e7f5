"""Host data projected with the sinogram streamed in angle chunks
(tsgb_direct_fp_angles, tsgb_direct_bp_angles, tsgb_copy_sino_angles).

The forward projection equals the one-call device path bit for bit; the
matched backprojection, accumulated chunk by chunk, equals it up to fp32
summation order. The size threshold is lowered so a small case streams.
"""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300 import _native, projector as projector_mod
from tests.helpers import TOL_ADJOINT, noise_cube_phantom, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture
def dev(native_lib, monkeypatch):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    monkeypatch.setattr(projector_mod, "PIPELINE_MIN_BYTES", 0)
    calls = []
    real = projector_mod._project_pipelined
    monkeypatch.setattr(projector_mod, "_project_pipelined",
                        lambda *a, **k: (calls.append(a[1]), real(*a, **k))[1])
    return torch.device("cuda", 0), calls


@pytest.mark.parametrize("geom", ["cone", "parallel_tilted"])
def test_streamed_host_projection_matches_device(dev, geom):
    dev, calls = dev
    vg = ts.volume(shape=(24, 28, 32), size=1)
    if geom == "cone":
        pg = ts.cone(angles=40, shape=(30, 44), size=1.5, cone_angle=0.4)
    else:  # general backprojection angles too
        R = ts.rotate(pos=0, axis=(1.0, 0.4, -0.3), angles=0.5)
        pg = R * ts.parallel(angles=33, shape=(30, 44), size=1.6).to_vec()
    A = ts.operator(vg, pg)
    x = noise_cube_phantom(vg.shape, seed=3)
    y_dev = A(torch.from_numpy(x).to(dev)).cpu().numpy()
    y_host = A(x)  # numpy in, numpy out: streamed
    assert np.array_equal(y_host, y_dev)
    xh = torch.from_numpy(x).pin_memory()
    yh = torch.zeros(A.range_shape, dtype=torch.float32).pin_memory()
    A(xh, out=yh)  # pinned tensors: streamed asynchronously
    assert np.array_equal(yh.numpy(), y_dev)
    ts.operator(vg, pg, additive=True)(xh, out=yh)
    assert np.array_equal(yh.numpy(), 2 * y_dev)
    bp_dev = A.T(torch.from_numpy(y_dev).to(dev)).cpu().numpy()
    bp_host = A.T(y_dev)
    assert rel_l2(bp_host, bp_dev) <= TOL_ADJOINT
    vh = torch.from_numpy(bp_host.copy()).pin_memory()
    ts.operator(vg, pg, additive=True).T(torch.from_numpy(y_dev).pin_memory(), out=vh)
    assert rel_l2(vh.numpy(), 2 * bp_dev) <= TOL_ADJOINT
    assert calls == [True, True, True, False, False]


def test_angle_range_arguments_are_checked(dev):
    dev, _ = dev
    A = ts.operator(ts.volume(shape=8, size=1), ts.cone(angles=6, shape=(8, 8), cone_angle=0.3))
    h = A.projector.handle(dev.index)
    lib = _native.load()
    x = torch.zeros(A.domain_shape, device=dev)
    y = torch.zeros(A.range_shape, device=dev)
    ws = torch.empty(A.projector.workspace_bytes(dev.index, True), dtype=torch.uint8, device=dev)
    for a0, a1 in ((3, 3), (-1, 2), (4, 7)):
        rc = lib.tsgb_direct_fp_angles(h, x.data_ptr(), y.data_ptr(), 0, a0, a1, 0, ws.data_ptr(),
                                       ws.numel(), None)
        assert rc == -1
    assert lib.tsgb_copy_sino_angles(None, None, 8, 6, 8, 0, 1, None) == -1
    B = ts.operator(ts.volume(shape=8, size=1), ts.cone(angles=6, shape=(8, 8), cone_angle=0.3),
                    detector_supersampling=2)
    rc = lib.tsgb_direct_fp_angles(B.projector.handle(dev.index), x.data_ptr(), y.data_ptr(), 0,
                                   0, 2, 0, ws.data_ptr(), ws.numel(), None)
    assert rc == -1 and b"supersampling" in lib.tsgb_last_error()
