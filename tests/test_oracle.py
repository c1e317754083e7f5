"""The FP64 oracle against known answers, exact identities of the
discretisation, the reference's one numeric output and the committed golden
fixtures; and the FDK oracle against a known reconstruction (CPU only)."""
import json
import os

import numpy as np
import pytest

import tomosipo_gb300 as ts
from oracle import oracle as orc
from tests.helpers import adjoint_error, ellipsoid_phantom, rel_l2

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_parallel_chord_length_unit_cube():
    # A ray along an axis through a unit cube of ones integrates to 1.0.
    vg = ts.volume(shape=16, size=1)
    pg = ts.parallel(angles=[0.0, np.pi / 2], shape=(16, 24), size=(1, 1.5))
    y = orc.fp(vg, pg, np.ones(vg.shape))
    inside = y[:, :, 4:20]
    assert np.allclose(inside, 1.0)
    assert np.allclose(y[:, :, :3], 0.0) and np.allclose(y[:, :, 21:], 0.0)


def test_parallel_diagonal_chord():
    # At 45 degrees a ray at perpendicular offset d from the centre has chord sqrt2 - 2d.
    n = 64
    vg = ts.volume(shape=(1, n, n), size=(1.0 / n, 1, 1))
    pg = ts.parallel(angles=[np.pi / 4], shape=(1, 2 * n), size=(1.0 / n, 2.0))
    y = orc.fp(vg, pg, np.ones(vg.shape))[0, 0]
    su = 2.0 / (2 * n)
    for iu in range(n - 8, n + 8):
        d = abs((iu + 0.5 - n) * su)
        assert y[iu] == pytest.approx(np.sqrt(2) - 2 * d, abs=2e-3)


def test_cone_central_ray_chord():
    # The cone ray through the volume centre along an axis has chord = volume size.
    vg = ts.volume(shape=16, size=1)
    pg = ts.cone(angles=[0.0], shape=(15, 15), size=1.5, src_orig_dist=3, src_det_dist=4)
    y = orc.fp(vg, pg, np.ones(vg.shape))
    assert y[7, 0, 7] == pytest.approx(1.0, abs=1e-12)


def test_parallel_opposite_angles_see_a_mirrored_detector():
    # At theta + pi the same rays run backwards and det_u flips (tomosipo's
    # parallel.to_vec): sinogram column u there is column C - 1 - u at theta.
    vg = ts.volume(shape=(8, 12, 12), size=(8 / 12, 1, 1))
    pg = ts.parallel(angles=[0.3, 0.3 + np.pi], shape=(8, 16), size=(8 / 12, 1.4))
    y = orc.fp(vg, pg, np.random.default_rng(7).random(vg.shape))
    assert np.abs(y[:, 1, :] - y[:, 0, ::-1]).max() < 1e-12


@pytest.mark.parametrize("cone", [False, True])
def test_rotating_the_volume_is_advancing_the_angle(cone):
    # Rotating the volume by a quarter turn in the (y, x) plane (np.rot90 over
    # axes y, x) and projecting at theta equals projecting the original at
    # theta + pi/2: pins the direction in which angles turn the source and
    # detector, for both beam types.
    vg = ts.volume(shape=(8, 12, 12), size=(8 / 12, 1, 1))
    x = np.random.default_rng(7).random(vg.shape)

    def geometry(theta):
        if cone:
            return ts.cone(angles=[theta], shape=(8, 16), size=(8 / 12, 1.4),
                           src_orig_dist=3, src_det_dist=5)
        return ts.parallel(angles=[theta], shape=(8, 16), size=(8 / 12, 1.4))

    rotated = np.ascontiguousarray(np.rot90(x, k=1, axes=(1, 2)))
    a = orc.fp(vg, geometry(0.2), rotated)
    assert np.abs(a - orc.fp(vg, geometry(0.2 + np.pi / 2), x)).max() < 1e-12
    assert np.abs(a - orc.fp(vg, geometry(0.2 - np.pi / 2), x)).max() > 1e-2


@pytest.mark.parametrize("dz, dx", [(0, 3), (2, 0), (1, -2)])
def test_moving_the_volume_by_whole_voxels_shifts_the_sinogram(dz, dx):
    # Parallel beam at theta = 0 (det_v along z, det_u along x) with pixel
    # pitch = voxel pitch: moving the volume by whole voxels shifts the
    # sinogram by as many pixels (the shadow stays on the detector).
    x = np.random.default_rng(3).random((6, 10, 10))
    pg = ts.parallel(angles=[0.0], shape=(12, 20), size=(1.2, 2.0))
    y = orc.fp(ts.volume(shape=(6, 10, 10), size=(0.6, 1, 1)), pg, x)
    moved = ts.volume(shape=(6, 10, 10), size=(0.6, 1, 1), pos=(0.1 * dz, 0, 0.1 * dx))
    expected = np.roll(np.roll(y, dz, axis=0), dx, axis=2)
    assert np.abs(orc.fp(moved, pg, x) - expected).max() < 1e-12


@pytest.mark.parametrize("cone", [False, True])
def test_scaling_the_whole_geometry_scales_the_integrals(cone):
    # World units: scaling volume, detector and distances by s scales every
    # line integral (FP) and every backprojected value (matched BP) by s.
    s = 2.5
    x = np.random.default_rng(3).random((6, 10, 10))

    def geometries(f):
        vg = ts.volume(shape=(6, 10, 10), size=(0.6 * f, f, f))
        if cone:
            return vg, ts.cone(angles=5, shape=(12, 20), size=(1.2 * f, 2.0 * f),
                               src_orig_dist=3 * f, src_det_dist=5 * f)
        return vg, ts.parallel(angles=5, shape=(12, 20), size=(1.2 * f, 2.0 * f))

    y = orc.fp(*geometries(1), x)
    assert np.abs(orc.fp(*geometries(s), x) - s * y).max() < 1e-12
    b = orc.bp_matched(*geometries(1), y)
    assert np.abs(orc.bp_matched(*geometries(s), y) - s * b).max() < 1e-12


@pytest.mark.parametrize("cone", [False, True])
def test_oracle_adjoint(cone):
    vg = ts.volume(shape=(12, 14, 16), size=(1, 1.2, 1.1))
    pg = (
        ts.cone(angles=9, shape=(13, 17), size=2, src_orig_dist=3, src_det_dist=4)
        if cone
        else ts.parallel(angles=9, shape=(13, 17), size=2)
    )
    rng = np.random.default_rng(1)
    x = rng.random(vg.shape)
    y = rng.random((13, 9, 17))
    for ss in (1, 2):
        Ax = orc.fp(vg, pg, x, det_ss=ss)
        ATy = orc.bp_matched(vg, pg, y, det_ss=ss)
        assert adjoint_error(Ax, y, x, ATy) < 1e-13


@pytest.mark.parametrize("cone,band", [(False, 0.03), (True, 0.2)])
def test_bilinear_approximates_matched(cone, band):
    """The bilinear backprojector approximates the transpose: equal totals (both
    spread each ray's value over voxel volume / pixel area), and close values.
    In cone beams the matched transpose aliases where rays are sparser than
    voxels (beyond the detector plane here), hence the wider band."""
    vg = ts.volume(shape=32, size=1)
    pg = (
        ts.cone(angles=32, shape=(32, 48), size=np.sqrt(2), cone_angle=0.5)
        if cone
        else ts.parallel(angles=32, shape=(32, 48), size=(1, 1.5))
    )
    x = ellipsoid_phantom(vg.shape, n=6, seed=2).astype(np.float64)
    y = orc.fp(vg, pg, x)
    bb, bm = orc.bp_bilinear(vg, pg, y), orc.bp_matched(vg, pg, y)
    assert bb.sum() == pytest.approx(bm.sum(), rel=1e-3)
    assert rel_l2(bb, bm) < band


@pytest.mark.parametrize("cone", [False, True])
def test_detector_supersampling_is_binned_fine_detector(cone):
    """d x d rays per pixel == the plain projection onto a d-times finer detector,
    averaged over d x d blocks (exact identity of the discretisation)."""
    vg = ts.volume(shape=(12, 14, 16), size=1)
    pg = (
        ts.cone(angles=5, shape=(9, 11), size=(1.3, 1.7), src_orig_dist=3, src_det_dist=4)
        if cone
        else ts.parallel(angles=5, shape=(9, 11), size=(1.3, 1.7))
    )
    x = np.random.default_rng(4).random(vg.shape)
    for d in (2, 3):
        fine = orc.fp(vg, pg.to_vec().reshape((9 * d, 11 * d)), x)
        binned = fine.reshape(9, d, 5, 11, d).mean(axis=(1, 4))
        assert rel_l2(orc.fp(vg, pg, x, det_ss=d), binned) < 1e-12


@pytest.mark.parametrize("cone", [False, True])
def test_voxel_supersampling_is_a_summed_fine_volume(cone):
    """The bilinear BP with d^3 points per voxel == the plain bilinear BP onto
    a d-times finer volume (each fine voxel weighted by its own volume),
    summed over d x d x d blocks (exact identity of the discretisation)."""
    box = dict(size=(0.6, 0.7, 0.8), pos=(0.02, -0.03, 0.01))
    vg = ts.volume(shape=(6, 7, 8), **box)
    pg = (
        ts.cone(angles=5, shape=(9, 11), size=(1.3, 1.7), src_orig_dist=3, src_det_dist=4)
        if cone
        else ts.parallel(angles=5, shape=(9, 11), size=(1.3, 1.7))
    )
    y = np.random.default_rng(5).random((9, 5, 11))
    for d in (2, 3):
        fine = orc.bp_bilinear(ts.volume(shape=(6 * d, 7 * d, 8 * d), **box), pg, y)
        summed = fine.reshape(6, d, 7, d, 8, d).sum(axis=(1, 3, 5))
        assert rel_l2(orc.bp_bilinear(vg, pg, y, vox_ss=d), summed) < 1e-12


def test_reference_notebook_hollow_box_pin():
    """notebooks/cupy.ipynb cell 4 (reference, ASTRA on GPU): hollow box on a 128^3
    unit cube, ts.parallel(angles=180, shape=128): sinogram mean 0.109146185,
    max 0.8471311. The old-API detector size is not printed; size sqrt(2) is the
    one consistent with the mean. The mean depends only on the world-unit scaling
    (line integrals / pixel area), the max also on the interpolation (ASTRA uses
    fixed-point texture weights), so it gets the 5e-3 ASTRA band."""
    with open(os.path.join(GOLDEN, "reference_pins.json")) as f:
        pin = json.load(f)["cupy_notebook_hollow_box"]
    vg = ts.volume(shape=128, size=1)
    x = np.zeros(vg.shape)
    ts.phantom.hollow_box(x)
    assert x.mean() == pytest.approx(pin["volume_mean"], rel=1e-6)
    pg = ts.parallel(angles=180, shape=128, size=np.sqrt(2))
    y = orc.fp(vg, pg, x)
    assert y.mean() == pytest.approx(pin["sino_mean"], rel=1e-4)
    assert y.max() == pytest.approx(pin["sino_max"], rel=5e-3)


def _golden_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("name", sorted(_golden_cases()))
def test_oracle_matches_golden_fixture(name):
    from tests.golden.make_golden import build_case

    vg, pg, x, y = build_case(name)
    data = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    assert rel_l2(orc.fp(vg, pg, x), data["fp"]) < 1e-12
    assert rel_l2(orc.bp_matched(vg, pg, y), data["bp_matched"]) < 1e-12
    assert rel_l2(orc.bp_bilinear(vg, pg, y), data["bp_bilinear"]) < 1e-12


def test_fdk_oracle_reconstructs_a_ball():
    """The NumPy FDK oracle (oracle/fdk_oracle.py) on the FP64 oracle's
    projections of a uniform ball (full circular cone scan, 120 angles):
    FDK's near-exact region recovers the density (measured: interior mean
    0.9994, worst interior voxel 1.75 % off, outside mean 0.004)."""
    from oracle import fdk_oracle

    n = 32
    vg = ts.volume(shape=n, size=1)
    pg = ts.cone(angles=120, shape=(48, 48), size=1.6, src_orig_dist=3, src_det_dist=4.5)
    g = (np.arange(n) + 0.5) / n - 0.5
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    r2 = Z ** 2 + Y ** 2 + X ** 2
    rec = fdk_oracle.fdk(vg, pg, orc.fp(vg, pg, (r2 < 0.3 ** 2).astype(np.float64)))
    inner, outer = r2 < 0.2 ** 2, r2 > 0.4 ** 2
    assert abs(rec[inner].mean() - 1) < 0.01 and np.abs(rec[inner] - 1).max() < 0.03
    assert abs(rec[outer].mean()) < 0.02


def test_oracle_results_do_not_depend_on_the_thread_count():
    # The golden fixtures are reproducible on any host only if this holds:
    # every voxel / pixel is summed by one thread in a fixed order.
    from tests.golden.make_golden import build_case

    vg, pg, x, y = build_case("cone_vec_helical")
    for f, arg in ((orc.fp, x), (orc.bp_matched, y), (orc.bp_bilinear, y)):
        one = f(vg, pg, arg, threads=1)
        for t in (3, 8):
            assert np.array_equal(f(vg, pg, arg, threads=t), one), (f.__name__, t)
