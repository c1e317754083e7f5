"""FDK (tomosipo's fdk, tomosipo/astra.py:374-406) and the legacy projection
functions on the GPU.

Parity: the GPU FDK against the FP64 NumPy FDK (oracle/fdk_oracle.py) on the
same sinogram, relative L2 <= 1e-5 (TOL_ORACLE; the GPU filters in fp32 with
an FFT, the oracle convolves in fp64). Physics: FDK of a full-circle cone scan
of a smooth phantom reproduces it in the central slab.
"""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from oracle import fdk_oracle
from tests.helpers import TOL_ORACLE, ellipsoid_phantom, helical_cone_vec, rel_l2
from tomosipo_gb300.astra import backward, fdk, forward
from tomosipo_gb300.fdk import fdk_reconstruct

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


CASES = {
    "cone": (ts.volume(shape=24, size=1), ts.cone(angles=40, shape=(24, 36), size=np.sqrt(2), cone_angle=0.5)),
    # the benchmark's cone family (unit cube, sqrt(2) detector, cone angle 0.5)
    # at 64^3, 64 angles, 64 x 96
    "cone_64_benchmark_family": (
        ts.volume(shape=64, size=1),
        ts.cone(angles=64, shape=(64, 96), size=np.sqrt(2), cone_angle=0.5),
    ),
    "cone_aniso_offset": (
        ts.volume(shape=(20, 24, 28), size=(0.8, 1.0, 1.1), pos=(0.02, -0.05, 0.04)),
        ts.cone(angles=30, shape=(22, 40), size=(1.2, 2.0), src_orig_dist=3.0, src_det_dist=4.5),
    ),
    "cone_vec_helical": (
        ts.volume(shape=20, size=1),
        helical_cone_vec(48, (24, 36), (1.0, 1.6), 2.5, 1.0, pitch=0.2, turns=1.0, jitter=0.3,
                         voxel=1 / 20),
    ),
    # a scan about a tilted axis: every angle's projection depends on z, so the
    # general bilinear kernel backprojects
    "cone_rotated": (
        ts.volume(shape=20, size=1),
        ts.rotate(pos=0, axis=(1.0, 0.3, -0.2), angles=0.4)
        * ts.cone(angles=36, shape=(24, 36), size=np.sqrt(2), cone_angle=0.5).to_vec(),
    ),
    # pi + 0.8 rad, with Parker's weights (fan half-angle about 0.34 rad)
    "cone_short_scan": (
        ts.volume(shape=20, size=1),
        ts.cone(angles=np.linspace(0, np.pi + 0.8, 36, endpoint=False), shape=(24, 36),
                size=np.sqrt(2), cone_angle=0.5),
    ),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fdk_matches_fp64_oracle(dev, name):
    vg, pg = CASES[name]
    short = name == "cone_short_scan"
    rng = np.random.default_rng(4)
    y = rng.random((pg.det_shape[0], pg.num_angles, pg.det_shape[1])).astype(np.float32)
    x_gpu = fdk_reconstruct(vg, pg, torch.from_numpy(y).to(dev), short_scan=short).cpu().numpy()
    x_ref = fdk_oracle.fdk(vg, pg, y, short_scan=short)
    assert rel_l2(x_gpu, x_ref) <= TOL_ORACLE, rel_l2(x_gpu, x_ref)


def test_fdk_short_scan_reconstructs_a_phantom(dev):
    """A scan of pi plus the fan angle: with Parker's weights FDK recovers the
    phantom about as well as from a full circle; without them the doubly
    measured lines bias it."""
    vg = ts.volume(shape=64, size=1)
    kw = dict(shape=(96, 96), size=np.sqrt(2) * 1.2, cone_angle=0.3)
    # pi + 0.7 rad: the detector's fan half-angle is below 0.2 rad
    pg = ts.cone(angles=np.linspace(0, np.pi + 0.7, 120, endpoint=False), **kw)
    A = ts.operator(vg, pg)
    x = torch.from_numpy(ellipsoid_phantom(vg.shape, n=6, seed=3)).to(dev)
    y = A(x)
    mid = slice(24, 40)
    ref = x[mid].cpu().numpy()
    err_parker = rel_l2(fdk_reconstruct(vg, pg, y, short_scan=True)[mid].cpu().numpy(), ref)
    err_plain = rel_l2(fdk_reconstruct(vg, pg, y)[mid].cpu().numpy(), ref)
    full = ts.cone(angles=180, **kw)
    err_full = rel_l2(fdk_reconstruct(vg, full, ts.operator(vg, full)(x))[mid].cpu().numpy(), ref)
    assert err_parker < 0.3 and err_parker < 0.6 * err_plain, (err_parker, err_plain)
    assert err_parker < 1.5 * err_full, (err_parker, err_full)


def test_fdk_of_a_rotated_scan_reconstructs_a_phantom(dev):
    """The same scan about a tilted axis reconstructs the rotated phantom as
    well as the upright scan reconstructs the upright one (general kernel)."""
    vg = ts.volume(shape=48, size=1)
    pg = ts.cone(angles=120, shape=(72, 72), size=np.sqrt(2) * 1.2, cone_angle=0.3)
    R = ts.rotate(pos=0, axis=(1.0, 0.2, 0.1), angles=0.3)
    x = torch.from_numpy(ellipsoid_phantom(vg.shape, n=6, seed=5)).to(dev)
    # the rotated scan of the phantom equals the upright scan of the inversely
    # rotated volume; compare both reconstructions in their own frames
    A_rot = ts.operator(vg, R * pg.to_vec())
    rec_rot = fdk_reconstruct(vg, R * pg.to_vec(), A_rot(x))
    rec = fdk_reconstruct(vg, pg, ts.operator(vg, pg)(x))
    mid = slice(18, 30)
    ref = x[mid].cpu().numpy()
    e_rot = rel_l2(rec_rot[mid].cpu().numpy(), ref)
    e = rel_l2(rec[mid].cpu().numpy(), ref)
    assert e_rot < 0.3 and e_rot < 1.5 * e, (e_rot, e)


def test_fdk_reconstructs_a_phantom(dev):
    vg = ts.volume(shape=64, size=1)
    pg = ts.cone(angles=180, shape=(96, 96), size=np.sqrt(2) * 1.2, cone_angle=0.3)
    A = ts.operator(vg, pg)
    x = torch.from_numpy(ellipsoid_phantom(vg.shape, n=6, seed=3)).to(dev)
    rec = fdk_reconstruct(vg, pg, A(x))
    mid = slice(24, 40)
    err = rel_l2(rec[mid].cpu().numpy(), x[mid].cpu().numpy())
    assert err < 0.25, err  # FDK on a 64^3 grid: blur at edges, small cone artefacts
    assert abs(float(rec[mid].mean()) / float(x[mid].mean()) - 1) < 0.03


def test_legacy_fdk_accumulates_and_forward_backward_match_operator(dev):
    pg = ts.cone(size=np.sqrt(2), cone_angle=1 / 2, angles=40, shape=32)
    vg = ts.volume(shape=32)
    pd = ts.data(pg)
    vd = ts.data(vg)
    vd.data[:] = ellipsoid_phantom(vg.shape, n=5, seed=1)
    x0 = vd.data.copy()
    forward(vd, pd)
    A = ts.operator(vg, pg)
    assert rel_l2(pd.data, A(x0)) < 1e-6
    rec = fdk_reconstruct(vg, pg, torch.from_numpy(pd.data).to(dev)).cpu().numpy()
    fdk(vd, pd)  # accumulates, as ASTRA's accumulate_FDK
    assert rel_l2(vd.data, x0 + rec) < 1e-6
    vd2 = ts.data(vg)
    backward(vd2, pd)
    assert rel_l2(vd2.data, A.T(pd.data)) < 1e-6


def test_composite_projection_sums_volumes(dev):
    pg = ts.cone(angles=12, shape=(16, 20), size=1.4, cone_angle=0.4)
    vg = ts.volume(shape=16, size=1)
    a, b = ts.data(vg, ellipsoid_phantom(vg.shape, n=3, seed=2)), ts.data(vg, ellipsoid_phantom(vg.shape, n=3, seed=3))
    pd = ts.data(pg)
    forward(a, b, pd)
    A = ts.operator(vg, pg)
    assert rel_l2(pd.data, A(a.data) + A(b.data)) < 1e-6
    # detector and voxel supersampling keyword arguments are accepted (reference test_astra.py)
    for kw in (dict(detector_supersampling=2, voxel_supersampling=2), dict(detector_supersampling=2)):
        forward(a, pd, **kw)
        backward(a, pd, **kw)
