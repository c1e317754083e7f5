"""Parity of the sm_103a projector with the FP64 oracle, through the public API.

Every case runs forward projection, matched backprojection and bilinear
backprojection on the GPU (ts.operator -> C ABI -> kernels) and compares
them with the oracle on the same seeded inputs. Gates: relative L2 error
<= 1e-5 (TOL_ORACLE) and adjointness <= 1e-6 (TOL_ADJOINT).
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
    helical_cone_vec,
    noise_cube_phantom,
    rel_l2,
)

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(7)
    R = ts.rotate(pos=0, axis=rng.normal(size=3), angles=0.7)
    R2 = ts.rotate(pos=0, axis=(1.0, 0.3, -0.2), angles=0.4)
    vg32 = ts.volume(shape=32, size=1)
    return {
        "parallel": (vg32, ts.parallel(angles=24, shape=(32, 48), size=(1, 1.5))),
        "cone": (vg32, ts.cone(angles=24, shape=(32, 48), size=np.sqrt(2), cone_angle=0.5)),
        "parallel_aniso": (
            ts.volume(shape=(20, 28, 36), size=(0.7, 1.1, 1.3), pos=(0.05, -0.1, 0.2)),
            ts.parallel(angles=np.linspace(0.1, 3.0, 13), shape=(17, 29), size=(1.2, 2.1)),
        ),
        "cone_aniso": (
            ts.volume(shape=(20, 28, 36), size=(0.7, 1.1, 1.3), pos=(0.05, -0.1, 0.2)),
            ts.cone(angles=11, shape=(19, 31), size=(1.5, 2.5), src_orig_dist=3.0, src_det_dist=4.5),
        ),
        "cone_vec_helical": (
            vg32,
            helical_cone_vec(40, (24, 40), (1.0, 1.6), 2.5, 1.0, pitch=0.3, turns=1.5,
                             jitter=0.5, voxel=1 / 32),
        ),
        "parallel_vec_rotated": (vg32, R * ts.parallel(angles=16, shape=(40, 48), size=(1.4, 1.6)).to_vec()),
        "cone_vec_rotated": (
            vg32,
            R2 * ts.cone(angles=12, shape=(36, 44), size=1.6, src_orig_dist=2.5, src_det_dist=3.5).to_vec(),
        ),
        "parallel_45deg": (vg32, ts.parallel(angles=[np.pi / 4, 3 * np.pi / 4, 0.0], shape=(32, 48), size=(1, 1.5))),
        "one_angle_one_row": (vg32, ts.cone(angles=[0.3], shape=(1, 48), size=(0.1, 1.5), src_orig_dist=3, src_det_dist=3)),
        "small_detector": (vg32, ts.parallel(angles=9, shape=(8, 8), size=(0.3, 0.3))),
    }


CASES = _cases()
# matched backprojectors: voxel-pair threads (0) and z-lane warps (1)
BP_KERNELS = (0, 1)


@pytest.fixture(scope="module")
def device(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp_bp_parity(name, device):
    vg, pg = CASES[name]
    A = ts.operator(vg, pg)
    x = noise_cube_phantom(vg.shape, seed=11)
    y_gpu = A(torch.from_numpy(x).to(device)).cpu().numpy()
    y_ref = orc.fp(vg, pg, x)
    assert y_gpu.shape == y_ref.shape == A.range_shape
    assert rel_l2(y_gpu, y_ref) <= TOL_ORACLE, rel_l2(y_gpu, y_ref)

    rng = np.random.default_rng(12)
    yy = rng.random(A.range_shape).astype(np.float32)
    x_ref = orc.bp_matched(vg, pg, yy)
    for kernel in BP_KERNELS:  # both matched backprojectors
        A.projector.set_tuning(device.index, bp_kernel=kernel, bp_shape=0)
        x_gpu = A.T(torch.from_numpy(yy).to(device)).cpu().numpy()
        assert rel_l2(x_gpu, x_ref) <= TOL_ORACLE, (kernel, rel_l2(x_gpu, x_ref))
        assert adjoint_error(y_gpu, yy, x, x_gpu) <= TOL_ADJOINT, kernel

    B = ts.operator(vg, pg, backprojector="bilinear")
    xb_gpu = B.T(torch.from_numpy(yy).to(device)).cpu().numpy()
    xb_ref = orc.bp_bilinear(vg, pg, yy)
    assert rel_l2(xb_gpu, xb_ref) <= TOL_ORACLE, rel_l2(xb_gpu, xb_ref)


SS_CASES = {
    "cone_ss2": (ts.volume(shape=24, size=1),
                 ts.cone(angles=9, shape=(20, 30), size=np.sqrt(2), cone_angle=0.5), 2),
    "parallel_ss3": (ts.volume(shape=(16, 20, 24), size=(0.8, 1.0, 1.2)),
                     ts.parallel(angles=7, shape=(11, 17), size=(1.0, 1.7)), 3),
    "cone_vec_rotated_ss2": (
        ts.volume(shape=16, size=1),
        ts.rotate(pos=0, axis=(1.0, 0.3, -0.2), angles=0.4)
        * ts.cone(angles=5, shape=(14, 18), size=1.6, src_orig_dist=2.5, src_det_dist=3.5).to_vec(),
        2,
    ),
}


@pytest.mark.parametrize("name", sorted(SS_CASES))
def test_detector_supersampling_parity(name, device):
    """Detector supersampling d: FP averages d x d rays per pixel (oracle: the
    same sub-rays in fp64), the matched BP is its exact transpose, and the
    bilinear BP ignores it (as ASTRA's does: it supersamples voxels)."""
    vg, pg, d = SS_CASES[name]
    A = ts.operator(vg, pg, detector_supersampling=d)
    assert A.range_shape == ts.operator(vg, pg).range_shape
    x = noise_cube_phantom(vg.shape, seed=5)
    y_gpu = A(torch.from_numpy(x).to(device)).cpu().numpy()
    y_ref = orc.fp(vg, pg, x, det_ss=d)
    assert rel_l2(y_gpu, y_ref) <= TOL_ORACLE, rel_l2(y_gpu, y_ref)
    yy = np.random.default_rng(6).random(A.range_shape).astype(np.float32)
    x_gpu = A.T(torch.from_numpy(yy).to(device)).cpu().numpy()
    x_ref = orc.bp_matched(vg, pg, yy, det_ss=d)
    assert rel_l2(x_gpu, x_ref) <= TOL_ORACLE, rel_l2(x_gpu, x_ref)
    assert adjoint_error(y_gpu, yy, x, x_gpu) <= TOL_ADJOINT
    # additive forward projection on top of an existing sinogram
    y2 = torch.from_numpy(y_gpu).to(device)
    ts.operator(vg, pg, detector_supersampling=d, additive=True)(torch.from_numpy(x).to(device), out=y2)
    assert rel_l2(y2.cpu().numpy(), 2 * y_ref) <= TOL_ORACLE
    B = ts.operator(vg, pg, detector_supersampling=d, backprojector="bilinear")
    B1 = ts.operator(vg, pg, backprojector="bilinear")
    yt = torch.from_numpy(yy).to(device)
    assert torch.equal(B.T(yt), B1.T(yt))


def test_minimum_slice_parallel64(device):
    """Plain parallel3d: 64^3 unit cube, noise + unit cube, 96 angles, detector 64x96."""
    vg = ts.volume(shape=64, size=1)
    pg = ts.parallel(angles=96, shape=(64, 96), size=(1, 1.5))
    A = ts.operator(vg, pg)
    x = noise_cube_phantom(vg.shape, seed=0)
    y = A(torch.from_numpy(x).to(device))
    y_ref = orc.fp(vg, pg, x)
    assert rel_l2(y.cpu().numpy(), y_ref) <= TOL_ORACLE
    bp = A.T(y)
    bp_ref = orc.bp_matched(vg, pg, y.cpu().numpy())
    assert rel_l2(bp.cpu().numpy(), bp_ref) <= TOL_ORACLE
    rng = np.random.default_rng(3)
    yy = torch.from_numpy(rng.random(A.range_shape).astype(np.float32)).to(device)
    assert adjoint_error(y.cpu(), yy.cpu(), x, A.T(yy).cpu()) <= TOL_ADJOINT


def test_cone_256_subset_parity(device):
    """Cone 256^3 (size sqrt2, cone angle 0.5, detector 256x384) on 24 of 360 angles."""
    vg = ts.volume(shape=256, size=1)
    full = ts.cone(angles=360, shape=(256, 384), size=np.sqrt(2), cone_angle=0.5)
    pg = full[::15]
    A = ts.operator(vg, pg)
    x = ellipsoid_phantom(vg.shape, seed=1)
    y = A(torch.from_numpy(x).to(device)).cpu().numpy()
    y_ref = orc.fp(vg, pg, x)
    assert rel_l2(y, y_ref) <= TOL_ORACLE, rel_l2(y, y_ref)
    bp_ref = orc.bp_matched(vg, pg, y)
    for kernel in BP_KERNELS:
        A.projector.set_tuning(device.index, bp_kernel=kernel, bp_shape=0)
        bp = A.T(torch.from_numpy(y).to(device)).cpu().numpy()
        assert rel_l2(bp, bp_ref) <= TOL_ORACLE, (kernel, rel_l2(bp, bp_ref))


def _headline_volume(n, seed):
    """float32 U[0, 1) noise plus 1.0 on the central half cube, built without
    float64 intermediates (a 512^3 float64 volume is 1 GB)."""
    rng = np.random.default_rng(seed)
    x = rng.random((n, n, n), dtype=np.float32)
    x[n // 4:3 * n // 4, n // 4:3 * n // 4, n // 4:3 * n // 4] += 1.0
    return x


def test_cone_512_headline_parity(device):
    """The benchmark's own configuration: cone 512^3, ts.cone(size=sqrt2,
    cone_angle=0.5), 1024 angles, detector 512 x 768. The GPU runs the full
    1024-angle operator (its real launch shapes, strides and workspace); the
    FP64 oracle checks 16 of the angles (every 64th):
      * FP: those 16 angle slices of A(x);
      * matched and bilinear BP: A.T of a sinogram that is random on those 16
        angles and exactly zero on the other 1008 (zeros add nothing);
      * adjointness of the full operator pair.
    """
    n, nang = 512, 1024
    vg = ts.volume(shape=n, size=1)
    pg = ts.cone(angles=nang, shape=(512, 768), size=np.sqrt(2), cone_angle=0.5)
    sub = pg[::64]
    A = ts.operator(vg, pg)
    x = _headline_volume(n, seed=41)
    xd = torch.from_numpy(x).to(device)
    y = A(xd)
    y_sub = y[:, ::64].cpu().numpy()
    y_ref = orc.fp(vg, sub, x)
    assert rel_l2(y_sub, y_ref) <= TOL_ORACLE, rel_l2(y_sub, y_ref)

    rng = np.random.default_rng(42)
    yy_sub = rng.random((512, 16, 768), dtype=np.float32)
    yy = torch.zeros(A.range_shape, device=device)
    yy[:, ::64] = torch.from_numpy(yy_sub).to(device)
    bp_ref = orc.bp_matched(vg, sub, yy_sub)
    # the default matched backprojector at this size (z-lane warps), then the
    # voxel-pair kernel
    assert A.projector.get_tuning(device.index)["bp_kernel"] == 1
    for tuning in (dict(bp_kernel=1, bp_shape=2), dict(bp_kernel=0)):
        A.projector.set_tuning(device.index, **tuning)
        bp = A.T(yy).cpu().numpy()
        assert rel_l2(bp, bp_ref) <= TOL_ORACLE, (tuning, rel_l2(bp, bp_ref))
        # <A x, yy> = <x, A^T yy>: yy is zero off the 16 angles
        assert adjoint_error(y_sub, yy_sub, x, bp) <= TOL_ADJOINT, tuning
    del bp_ref
    B = ts.operator(vg, pg, backprojector="bilinear")
    bb = B.T(yy).cpu().numpy()
    bb_ref = orc.bp_bilinear(vg, sub, yy_sub)
    assert rel_l2(bb, bb_ref) <= TOL_ORACLE, rel_l2(bb, bb_ref)
    del y, yy, xd
    torch.cuda.empty_cache()


def test_additive_is_twice(device):
    """tests/test_Operator.py:35-49: applying an additive operator twice = 2 A(x)."""
    vg = ts.volume(shape=40)
    pg = ts.cone(size=np.sqrt(2) * 40, cone_angle=1 / 2, angles=30, shape=40)
    A = ts.operator(vg, pg, additive=False)
    B = ts.operator(vg, pg, additive=True)
    x = torch.zeros(A.domain_shape, device=device)
    ts.phantom.hollow_box(x)
    y = torch.zeros(A.range_shape, device=device)
    B(x, out=y)
    B(x, out=y)
    assert torch.allclose(2 * A(x), y, rtol=1e-6, atol=1e-6)
    v = torch.zeros(A.domain_shape, device=device)
    B.T(y, out=v)
    B.T(y, out=v)
    assert torch.allclose(2 * A.T(y), v, rtol=1e-6, atol=1e-5)


def test_numpy_and_torch_inputs_agree(device):
    """tests/test_Operator.py:15-32: the array type does not change the result."""
    vg = ts.volume(shape=48)
    pg = ts.cone(size=np.sqrt(2) * 48, cone_angle=1 / 2, angles=40, shape=48)
    A = ts.operator(vg, pg)
    x = np.zeros(A.domain_shape, dtype=np.float32)
    ts.phantom.hollow_box(x)
    y_np = A(x)
    y_t = A(torch.from_numpy(x).to(device)).cpu().numpy()
    assert isinstance(y_np, np.ndarray)
    assert np.abs(y_np - y_t).sum() == pytest.approx(0.0)
    assert np.abs(A.T(y_np) - A.T(torch.from_numpy(y_t).to(device)).cpu().numpy()).sum() == pytest.approx(0.0, abs=1e-3)


def test_wide_sinogram_paths_by_linearity(device):
    """Maximum sizes: a sinogram of more than 2^31 detector pixels (with padding)
    takes the 64-bit-offset paths of the forward projector's output, the row-pair
    backprojector and the general bilinear backprojector. Splitting the angles in
    two halves gives operators below that size (32-bit paths): the forward
    projections must agree bit for bit per angle, and the backprojection must be
    the sum of the halves' within TOL_ORACLE. The two sums add the same ~12,000
    fp32 terms per voxel in different orders, which alone differs by ~2e-6; an
    offset error would be of order one."""
    vg = ts.volume(shape=32, size=1)
    pg = ts.cone(angles=2048, shape=(1024, 1040), size=1.5, cone_angle=0.3)
    rows, cols = pg.det_shape
    assert (rows + 4) * pg.num_angles * cols >= 2 ** 31
    A = ts.operator(vg, pg)
    A1, A2 = ts.operator(vg, pg[:1024]), ts.operator(vg, pg[1024:])
    x = torch.from_numpy(noise_cube_phantom(vg.shape, seed=9)).to(device)
    y = A(x)
    assert torch.equal(y[:, :1024], A1(x)) and torch.equal(y[:, 1024:], A2(x))
    bp = A.T(y)
    bp_split = A1.T(y[:, :1024].contiguous()) + A2.T(y[:, 1024:].contiguous())
    assert rel_l2(bp.cpu().numpy(), bp_split.cpu().numpy()) <= TOL_ORACLE
    B, B1, B2 = (ts.operator(vg, g, backprojector="bilinear") for g in (pg, pg[:1024], pg[1024:]))
    bb = B.T(y)
    bb_split = B1.T(y[:, :1024].contiguous()) + B2.T(y[:, 1024:].contiguous())
    assert rel_l2(bb.cpu().numpy(), bb_split.cpu().numpy()) <= TOL_ORACLE
    del y, bp, bb
    torch.cuda.empty_cache()


BP_EDGE_CASES = {
    # detector columns ~4x finer than voxels: many columns reach each voxel
    "fine_columns": (ts.volume(shape=(20, 24, 40), size=(0.5, 0.6, 1.0)),
                     ts.cone(angles=10, shape=(20, 240), size=(0.7, 1.6), cone_angle=0.3)),
    # detector rows ~3x finer than voxels along z: several rows per voxel
    # (the backprojector's row-loop path)
    "fine_rows": (ts.volume(shape=24, size=1),
                  ts.parallel(angles=12, shape=(80, 36), size=(1.2, 1.5))),
    # rows 2/3 of a voxel apart: up to four rows per voxel (the voxel-pair
    # kernel's four-row path; projectors with rows this fine use that kernel)
    "rows_finer_than_voxels": (ts.volume(shape=24, size=1),
                               ts.parallel(angles=12, shape=(36, 36), size=(1.0, 1.5))),
    # a detector shorter than the volume: rows clamped into the padding
    "tall_volume": (ts.volume(shape=(150, 20, 36), size=(3.0, 0.4, 0.72)),
                    ts.cone(angles=9, shape=(40, 50), size=(1.2, 1.0), src_orig_dist=3,
                            src_det_dist=4)),
}


@pytest.mark.parametrize("name", sorted(BP_EDGE_CASES))
def test_matched_bp_edge_geometries(name, device):
    """Matched backprojection against the oracle where detector sampling is
    much finer than the voxels (along u or v) or the detector is shorter than
    the volume, with adjointness and the additive form."""
    vg, pg = BP_EDGE_CASES[name]
    A = ts.operator(vg, pg)
    x = noise_cube_phantom(vg.shape, seed=21)
    y_gpu = A(torch.from_numpy(x).to(device)).cpu().numpy()
    assert rel_l2(y_gpu, orc.fp(vg, pg, x)) <= TOL_ORACLE
    yy = np.random.default_rng(22).random(A.range_shape).astype(np.float32)
    yt = torch.from_numpy(yy).to(device)
    x_ref = orc.bp_matched(vg, pg, yy)
    for kernel in BP_KERNELS:
        A.projector.set_tuning(device.index, bp_kernel=kernel, bp_shape=0)
        xb = A.T(yt)
        assert rel_l2(xb.cpu().numpy(), x_ref) <= TOL_ORACLE, (kernel, rel_l2(xb.cpu().numpy(), x_ref))
        assert adjoint_error(y_gpu, yy, x, xb.cpu().numpy()) <= TOL_ADJOINT, kernel
        acc = xb.clone()
        B = ts.operator(vg, pg, additive=True)
        B.projector.set_tuning(device.index, bp_kernel=kernel, bp_shape=0)
        B.T(yt, out=acc)
        assert rel_l2(acc.cpu().numpy(), 2 * x_ref) <= TOL_ORACLE, kernel


@pytest.mark.parametrize("d", [2, 3])
def test_voxel_supersampling_bilinear_parity(d, device):
    """voxel_supersampling d: the bilinear backprojection averages d^3 points
    per voxel (the oracle evaluates the same points in fp64); the forward
    projection and the matched backprojection do not change."""
    vg = ts.volume(shape=(14, 18, 22), size=(0.7, 0.9, 1.1))
    pg = ts.cone(angles=7, shape=(20, 30), size=(1.2, 1.6), src_orig_dist=2.5, src_det_dist=3.5)
    A = ts.operator(vg, pg, voxel_supersampling=d, backprojector="bilinear")
    yy = np.random.default_rng(31).random(A.range_shape).astype(np.float32)
    yt = torch.from_numpy(yy).to(device)
    xb = A.T(yt).cpu().numpy()
    ref = orc.bp_bilinear(vg, pg, yy, vox_ss=d)
    assert rel_l2(xb, ref) <= TOL_ORACLE, rel_l2(xb, ref)
    assert rel_l2(xb, orc.bp_bilinear(vg, pg, yy)) > 10 * TOL_ORACLE  # it does change
    x = torch.from_numpy(noise_cube_phantom(vg.shape, seed=32)).to(device)
    M, M1 = ts.operator(vg, pg, voxel_supersampling=d), ts.operator(vg, pg)
    assert torch.equal(M(x), M1(x)) and torch.equal(M.T(yt), M1.T(yt))
