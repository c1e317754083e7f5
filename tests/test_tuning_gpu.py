"""Forward-projector schedules (tsgb_tuning) and the autotuner.

The schedule only orders independent tiles and both copy layouts feed the
same arithmetic, so every tuning must give bit-identical sinograms, on detectors whose sizes are not multiples of the
tile and with odd angle counts (ragged last patch, strip, group and pair).
"""
import ctypes

import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300 import _native
from tomosipo_gb300.autotune import autotune
from tests.helpers import helical_cone_vec

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TUNINGS = [
    dict(fp_patch_rows=1, fp_patch_cols=1, fp_group_pairs=1, fp_pair_layout=0),
    dict(fp_patch_rows=3, fp_patch_cols=5, fp_group_pairs=2, fp_pair_layout=1),
    dict(fp_patch_rows=2, fp_patch_cols=64, fp_group_pairs=7, fp_pair_layout=0),
    dict(fp_patch_rows=16, fp_patch_cols=3, fp_group_pairs=1000, fp_pair_layout=1),
]


def _geometries():
    vg = ts.volume(shape=(40, 33, 47), size=(1.0, 0.9, 1.2))
    return {
        "cone_ragged": (vg, ts.cone(angles=29, shape=(77, 45), size=(1.8, 2.0), cone_angle=0.4)),
        "parallel_ragged": (vg, ts.parallel(angles=31, shape=(70, 53), size=(1.6, 1.9))),
        "cone_vec_helical": (
            ts.volume(shape=32, size=1),
            helical_cone_vec(33, (40, 72), (1.0, 1.6), 2.5, 1.0, pitch=0.3, turns=1.5,
                             jitter=0.5, voxel=1 / 32),
        ),
        "one_angle": (vg, ts.cone(angles=[0.4], shape=(33, 17), size=(1.5, 1.5), cone_angle=0.3)),
    }


@pytest.fixture(scope="module")
def dev(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.mark.parametrize("name", sorted(_geometries()))
def test_every_schedule_gives_identical_sinograms(dev, name):
    vg, pg = _geometries()[name]
    A = ts.operator(vg, pg)
    g = torch.Generator(device="cpu").manual_seed(3)
    x = torch.rand(A.domain_shape, generator=g).to(dev)
    ref = A(x)
    default = A.projector.get_tuning(dev.index)
    for t in TUNINGS:
        A.projector.set_tuning(dev.index, **t)
        got = A.projector.get_tuning(dev.index)
        assert {k: got[k] for k in t} == t
        assert torch.equal(A(x), ref), t
        y = torch.ones_like(ref)
        A(x, out=y)
        assert torch.equal(y, ref)
    A.projector.set_tuning(dev.index, **default)


def test_set_tuning_rejects_bad_values(dev):
    A = ts.operator(ts.volume(shape=8, size=1), ts.cone(angles=3, shape=(8, 8), cone_angle=0.3))
    h = A.projector.handle(dev.index)
    lib = _native.load()
    for bad in (dict(fp_patch_rows=0), dict(fp_patch_cols=-1), dict(fp_group_pairs=0),
                dict(fp_pair_layout=2), dict(bp_kernel=2), dict(bp_shape=-1), dict(bp_shape=7),
                dict(bp_general=2), dict(bp_general=-1)):
        t = _native.Tuning(**dict(dict(fp_patch_rows=1, fp_patch_cols=1, fp_group_pairs=1), **bad))
        assert lib.tsgb_projector_set_tuning(h, ctypes.byref(t)) == -1
    t = _native.Tuning(fp_patch_rows=1, fp_patch_cols=1, fp_group_pairs=1)
    t.reserved = 1
    assert lib.tsgb_projector_set_tuning(h, ctypes.byref(t)) == -1
    with pytest.raises(ValueError):
        A.projector.set_tuning(dev.index, tile=3)


def test_autotune_keeps_results_and_caches(dev, tmp_path):
    vg, pg = _geometries()["cone_ragged"]
    A = ts.operator(vg, pg)
    x = torch.rand(A.domain_shape, device=dev)
    ref = A(x)
    path = str(tmp_path / "tuning.json")
    r = autotune(A, cache_path=path)
    assert not r["cached"] and r["trials"] > 1 and r["ms"] <= r["default_ms"]
    assert A.projector.get_tuning(dev.index) == r["tuning"]
    assert torch.equal(A(x), ref)
    B = ts.operator(vg, pg)  # same geometry, new projector: served from the cache
    r2 = autotune(B, cache_path=path)
    assert r2["cached"] and B.projector.get_tuning(dev.index) == r["tuning"]


BP_TUNINGS = [dict(bp_kernel=0, bp_shape=0)] + [dict(bp_kernel=1, bp_shape=k) for k in range(7)]


@pytest.mark.parametrize("name", sorted(_geometries()))
def test_every_backprojector_shape_agrees(dev, name):
    """The matched backprojection under every kernel and z-lane warp shape:
    the same sums in different orders (rel. L2 <= 1e-6 between them), each
    within the parity tolerance of the FP64 oracle, and additive mode adds."""
    from oracle import oracle as orc
    from tests.helpers import TOL_ORACLE, rel_l2

    vg, pg = _geometries()[name]
    A = ts.operator(vg, pg)
    B = ts.operator(vg, pg, additive=True)
    yy = torch.rand(A.range_shape, generator=torch.Generator().manual_seed(4)).to(dev)
    ref = orc.bp_matched(vg, pg, yy.cpu().numpy())
    default = A.projector.get_tuning(dev.index)
    first = None
    for t in BP_TUNINGS:
        A.projector.set_tuning(dev.index, **t)
        B.projector.set_tuning(dev.index, **t)
        got = A.T(yy)
        assert rel_l2(got.cpu().numpy(), ref) <= TOL_ORACLE, t
        first = got if first is None else first
        assert rel_l2(got.cpu().numpy(), first.cpu().numpy()) <= 1e-6, t
        acc = got.clone()
        B.T(yy, out=acc)
        assert rel_l2(acc.cpu().numpy(), 2 * ref) <= TOL_ORACLE, t
    A.projector.set_tuning(dev.index, **default)


def test_batched_sirt_follows_each_jobs_schedule(dev):
    from tomosipo_gb300.sirt import BatchedSirt, sirt

    vg = ts.volume(shape=(24, 20, 28), size=1)
    jobs = []
    for i, t in enumerate(TUNINGS[:3]):
        pg = ts.cone(angles=13 + 2 * i, shape=(37, 45), size=(1.5, 1.8), cone_angle=0.4)
        A = ts.operator(vg, pg)
        # jobs on both matched backprojectors (their residual layouts differ)
        A.projector.set_tuning(dev.index, **t, bp_kernel=i % 2)
        x = torch.rand(A.domain_shape, device=dev)
        jobs.append((A, A(x)))
    b = BatchedSirt(jobs)
    b.run(4, graph=False)
    for (A, y), xb in zip(jobs, b.x):
        assert torch.equal(xb, sirt(A, y, 4))
    b.close()
