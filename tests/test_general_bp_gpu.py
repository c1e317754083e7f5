"""The matched backprojection of angles outside the separable kernels (tilted
detectors, rotated scans): the box kernel, whose blocks stage each angle's
detector region in shared memory (tuning bp_general = 0, the default), against
one thread per voxel (bp_general = 1) and against the FP64 oracle.

Both kernels sum the same candidate pixels with the same weights in the same
order, so they agree to rounding-free equality except where a pixel's weight
is within a rounding step of zero; the gate between them is 1e-7 relative L2.
Cases cover both weighted-sinogram layouts (bp_kernel 0: row-major pairs,
1: column-major), the additive form, volumes that are not whole boxes, a scan
that mixes separable and tilted angles (the general kernel adds onto the
separable passes), and the box kernel's three ways of summing: a box-wide
window of candidate pixels (pixels about as large as voxels; unrolled sums for
windows of 3 x 2, 2 x 2, 3 x 3 and 2 x 3 pixels, loops for other shapes such
as 4 x 1 or 1 x 6, which the cases with oblong pixels reach), a bound per
voxel (footprints wider than that window), and, for a detector fine enough
that the staged region does not fit, the per-voxel sums.
"""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from oracle import oracle as orc
from tests.helpers import (
    TOL_ADJOINT,
    TOL_ORACLE,
    adjoint_error,
    ellipsoid_phantom,
    noise_cube_phantom,
    rel_l2,
)

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_KERNELS = 1e-7


def _cases():
    R = ts.rotate(pos=0, axis=(1.0, 0.3, -0.2), angles=0.4)
    R2 = ts.rotate(pos=0, axis=(0.2, 1.0, 0.5), angles=0.9)
    vg32 = ts.volume(shape=32, size=1)
    cone = ts.cone(angles=12, shape=(36, 44), size=1.6, src_orig_dist=2.5, src_det_dist=3.5)
    return {
        "cone_vec_tilted": (vg32, R * cone.to_vec()),
        "parallel_vec_tilted": (vg32, R2 * ts.parallel(angles=16, shape=(40, 48), size=(1.4, 1.6)).to_vec()),
        "ragged_volume": (
            ts.volume(shape=(20, 28, 37), size=(0.7, 1.1, 1.3), pos=(0.05, -0.1, 0.2)),
            R * ts.cone(angles=9, shape=(25, 41), size=(1.5, 2.5), src_orig_dist=3.0,
                        src_det_dist=4.5).to_vec(),
        ),
        "mixed_separable_and_tilted": (
            vg32, ts.concatenate([cone.to_vec()[:6], (R * cone.to_vec())[6:]])),
        # pixels ~2.5x finer than voxels: footprints wider than the box-wide
        # window, so each voxel bounds its own (the region still fits)
        "finer_detector_bounds": (
            ts.volume(shape=24, size=1),
            R * ts.cone(angles=5, shape=(60, 75), size=1.6, src_orig_dist=2.5,
                        src_det_dist=3.5).to_vec(),
        ),
        # pixels four times taller than wide (0.16 x 0.04 of a 24-voxel unit
        # volume): box-wide windows of 4 x 1, 4 x 2 and 3 x 1 pixels, which
        # take the window loops sized at run time
        "tall_pixel_windows": (
            ts.volume(shape=24, size=1),
            R * ts.cone(angles=5, shape=(10, 40), size=1.6, src_orig_dist=2.5,
                        src_det_dist=3.5).to_vec(),
        ),
        # pixels about four times wider than tall: windows of 1 x 5 and 1 x 6
        # pixels (wu * 4 + wv of a 1 x 6 window equals that of 2 x 2, so a
        # shape key of that form would sum the wrong window here)
        "wide_pixel_windows": (
            ts.volume(shape=24, size=1),
            R * ts.cone(angles=5, shape=(60, 14), size=1.6, src_orig_dist=2.5,
                        src_det_dist=3.5).to_vec(),
        ),
        # pixels ~4x finer than voxels: a box's region exceeds the stage
        "fine_detector_fallback": (
            ts.volume(shape=24, size=1),
            R * ts.cone(angles=5, shape=(120, 150), size=1.6, src_orig_dist=2.5,
                        src_det_dist=3.5).to_vec(),
        ),
    }


CASES = _cases()


@pytest.fixture(scope="module")
def device(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.mark.parametrize("name", sorted(CASES))
def test_box_kernel_equals_per_voxel_and_oracle(name, device):
    vg, pg = CASES[name]
    A = ts.operator(vg, pg)
    stats = A.projector.stats(device.index)
    assert stats["general_bp_angles"] > 0
    if name == "mixed_separable_and_tilted":
        assert stats["separable_bp_angles"] > 0
    x = noise_cube_phantom(vg.shape, seed=31)
    y = A(torch.from_numpy(x).to(device))
    yy = np.random.default_rng(32).random(A.range_shape).astype(np.float32)
    yt = torch.from_numpy(yy).to(device)
    x_ref = orc.bp_matched(vg, pg, yy)
    B = ts.operator(vg, pg, additive=True)
    for bp_kernel in (0, 1):  # row-major and column-major weighted sinograms
        out = {}
        for general in (0, 1):
            for op in (A, B):
                op.projector.set_tuning(device.index, bp_kernel=bp_kernel, bp_shape=0,
                                        bp_general=general)
            xb = A.T(yt)
            acc = xb.clone()
            B.T(yt, out=acc)
            out[general] = (xb, acc)
            err = rel_l2(xb.cpu().numpy(), x_ref)
            assert err <= TOL_ORACLE, (bp_kernel, general, err)
            assert adjoint_error(y.cpu().numpy(), yy, x, xb.cpu().numpy()) <= TOL_ADJOINT
            assert rel_l2(acc.cpu().numpy(), 2 * x_ref) <= TOL_ORACLE, (bp_kernel, general)
        for k in range(2):
            a, b = out[0][k].cpu().numpy(), out[1][k].cpu().numpy()
            assert rel_l2(a, b) <= TOL_KERNELS, (bp_kernel, k, rel_l2(a, b))
    A.projector.set_tuning(device.index, bp_general=0)


def test_box_kernel_in_batched_sirt_equals_plain(device):
    """Batched SIRT on a tilted scan runs the box kernel into its sum volume:
    bitwise equal to the plain loop, as with one thread per voxel."""
    from tomosipo_gb300.sirt import BatchedSirt, sirt

    vg, pg = CASES["cone_vec_tilted"]
    A = ts.operator(vg, pg)
    y = A(torch.from_numpy(noise_cube_phantom(vg.shape, seed=33)).to(device))
    for general in (0, 1):
        A.projector.set_tuning(device.index, bp_general=general)
        batch = BatchedSirt([(A, y)])
        batch.run(3, graph=False)
        assert torch.equal(batch.x[0], sirt(A, y, 3)), general
        batch.close()
    A.projector.set_tuning(device.index, bp_general=0)


def test_tilted_256_full_operator_subset_parity(device):
    """The benchmark's tilted scan at full size: cone 256^3, detector 256 x 384,
    360 angles, rotated 0.4 rad about (1, 0.3, -0.2), every angle on the
    general backprojector. The GPU runs the full 360-angle operator; the FP64
    oracle checks 12 of the angles (every 30th): FP slices, the box kernel's
    A.T of a sinogram that is zero off those angles, and adjointness."""
    n = 256
    vg = ts.volume(shape=n, size=1)
    R = ts.rotate(pos=0, axis=(1.0, 0.3, -0.2), angles=0.4)
    pg = R * ts.cone(angles=360, shape=(256, 384), size=np.sqrt(2), cone_angle=0.5).to_vec()
    sub = pg[::30]
    A = ts.operator(vg, pg)
    assert A.projector.stats(device.index)["general_bp_angles"] == 360
    assert A.projector.get_tuning(device.index)["bp_general"] == 0
    x = ellipsoid_phantom(vg.shape, seed=3)
    y = A(torch.from_numpy(x).to(device))
    y_sub = y[:, ::30].cpu().numpy()
    y_ref = orc.fp(vg, sub, x)
    assert rel_l2(y_sub, y_ref) <= TOL_ORACLE, rel_l2(y_sub, y_ref)
    yy_sub = np.random.default_rng(34).random((256, 12, 384), dtype=np.float32)
    yy = torch.zeros(A.range_shape, device=device)
    yy[:, ::30] = torch.from_numpy(yy_sub).to(device)
    bp = A.T(yy).cpu().numpy()
    bp_ref = orc.bp_matched(vg, sub, yy_sub)
    assert rel_l2(bp, bp_ref) <= TOL_ORACLE, rel_l2(bp, bp_ref)
    assert adjoint_error(y_sub, yy_sub, x, bp) <= TOL_ADJOINT
