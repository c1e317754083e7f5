"""Geometry API behaviour that tomosipo's own geometry tests pin
(``tests/geometry/test_parallel.py``, ``test_cone.py``, ``test_volume.py``,
``test_concatenate.py``), restated with seeded inputs: indexing rules, corners,
reshaping and rescaling, ASTRA round trips, transforms (with the warning when a
non-vector geometry becomes a vector one), ``project_point`` relations,
``to_vol``, volume operations and ``ts.concatenate``. Host only.
"""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300 import vector_calc as vc
from tomosipo_gb300.geometry import (
    random_cone,
    random_cone_vec,
    random_parallel,
    random_parallel_vec,
    random_transform,
    random_volume,
    random_volume_vec,
)
from tomosipo_gb300.geometry import transform


@pytest.fixture(autouse=True)
def _seeded():
    np.random.seed(123)  # the random_* helpers draw from NumPy's global generator


def _par_geoms():
    np.random.seed(7)
    return [ts.parallel(angles=2), ts.parallel(angles=10, size=3, shape=11),
            ts.parallel(angles=5, size=7, shape=23), random_parallel(), random_parallel()]


def _cone_geoms():
    np.random.seed(8)
    return [ts.cone(angles=3, cone_angle=0.5), ts.cone(angles=12, shape=(6, 10), size=(1.5, 2.5),
                                                      src_orig_dist=4, src_det_dist=6),
            random_cone(), random_cone()]


# ------------------------------------------------------------------ indexing
def test_parallel_getitem_rules():
    pg = ts.parallel(angles=10, shape=20)
    assert pg[1].num_angles == pg[:1].num_angles == pg[-1].num_angles == 1
    assert pg[:2].num_angles == 2 and pg[:].num_angles == 10
    assert pg[-1] == pg[9] and pg[-2] == pg[8]
    assert pg[np.ones(pg.num_angles) == 1] == pg
    assert pg[np.arange(pg.num_angles) % 2 == 0] == pg[0::2]
    with pytest.raises(ValueError):
        pg[:, 0, 0]  # no detector indexing on a non-vector geometry
    with pytest.raises(IndexError):
        ts.parallel(angles=3)[4]
    for g in _par_geoms():
        assert g == g[:]
        with pytest.raises(ValueError):
            g[:, :]
        assert g[1::2].num_angles == g.num_angles // 2
        assert g[1:9:2].angles == pytest.approx(g.angles[1:9:2])
        assert g[-1].angles == pytest.approx(g.angles[-1:])
        assert g[-2].angles == pytest.approx(g.angles[-2:-1])


def test_cone_getitem_rules():
    pg = ts.cone(angles=10, shape=20, cone_angle=0.5)
    assert pg[3].num_angles == 1 and pg[-1] == pg[9]
    assert pg[np.arange(10) % 3 == 0] == pg[0::3]
    with pytest.raises(ValueError):
        pg[:, 0, 0]


# ---------------------------------------------------------------- properties
@pytest.mark.parametrize("kind", ["parallel", "cone"])
def test_det_properties_and_corners(kind):
    for pg in (_par_geoms() if kind == "parallel" else _cone_geoms()):
        n = pg.num_angles
        for name in ("det_pos", "det_v", "det_u", "det_normal"):
            assert getattr(pg, name).shape == (n, 3), name
        assert pg.det_sizes.shape == (n, 2) and pg.corners.shape == (n, 4, 3)
        assert pg.lower_left_corner == pytest.approx(pg.corners[:, 0, :])
        half = pg.det_shape[0] * pg.det_v / 2 + pg.det_shape[1] * pg.det_u / 2
        assert pg.det_pos - pg.lower_left_corner == pytest.approx(half)
        assert pg.det_shape == pg.to_vec().det_shape and pg.num_angles == pg.to_vec().num_angles
        assert pg.det_sizes == pytest.approx(pg.to_vec().det_sizes)
        assert pg.det_pos == pytest.approx(pg.to_vol().pos)


def test_parallel_has_no_source():
    for pg in _par_geoms():
        assert pg.ray_dir.shape == (pg.num_angles, 3)
        with pytest.raises(NotImplementedError):
            pg.src_pos


def test_cone_distances_and_sizes():
    assert ts.cone(size=np.sqrt(2), src_orig_dist=5.0).src_orig_dist == 5.0
    assert ts.cone(size=np.sqrt(2), src_det_dist=3.0).src_det_dist == 3.0
    pg = ts.cone(angles=3, cone_angle=0.5, size=(1, 2))
    assert np.abs(pg.det_sizes - np.array([[1, 2]])).sum() < ts.epsilon


# -------------------------------------------------------- reshape and rescale
def test_reshape_keeps_detector_size():
    for pg in _par_geoms() + _cone_geoms():
        assert pg.reshape(1).det_shape == (1, 1)
        assert pg.reshape((3, 5)).det_shape == (3, 5)
        assert pg.reshape((3, 5)).det_sizes == pytest.approx(pg.det_sizes)


def test_rescale_det():
    for pg in _par_geoms():
        if pg.det_shape[0] % 2 == 0 and pg.det_shape[1] % 2 == 0:
            r = pg.rescale_det(2)
            assert r.angles == pytest.approx(pg.angles)
            assert r.det_shape == (pg.det_shape[0] // 2, pg.det_shape[1] // 2)
            assert r.det_sizes == pytest.approx(pg.det_sizes)
            assert r.det_v == pytest.approx(2 * pg.det_v)
            assert r.det_u == pytest.approx(2 * pg.det_u)
    pg = ts.cone(size=np.sqrt(2), cone_angle=0.5, angles=10, shape=20)
    assert pg.rescale_det(2).det_sizes == pytest.approx(pg.det_sizes)
    assert pg.rescale_det((2, 2)) == pg.rescale_det(2)
    assert pg.rescale_det(10).det_shape == (2, 2)


# ------------------------------------------------------------- ASTRA round trip
def test_astra_round_trips():
    for pg in _par_geoms() + _cone_geoms():
        assert pg == ts.from_astra(pg.to_astra())
        assert ts.from_astra(pg.to_vec().to_astra()) == ts.from_astra(pg.to_astra()).to_vec()
    rng = np.random.default_rng(9)
    for _ in range(20):
        n = int(rng.integers(1, 100))
        angles = rng.uniform(0, 2 * np.pi, n) if rng.random() < 0.5 else n
        pg = ts.cone(angles=angles, shape=rng.integers(1, 100, size=2), size=rng.uniform(1, 100, 2),
                     cone_angle=rng.uniform(0.5, 1))
        assert pg == ts.from_astra(pg.to_astra())


# ----------------------------------------------------------------- transforms
def test_transforms_compose_and_convert_with_a_warning():
    for pg in _par_geoms()[:3] + _cone_geoms()[:3]:
        T1, T2 = random_transform(), random_transform()
        with pytest.warns(UserWarning):
            assert (T1 * T2) * pg == T1 * (T2 * pg)
        with pytest.warns(UserWarning):
            assert transform.identity() * pg == pg.to_vec()
    for pg in (random_parallel_vec(), random_cone_vec()):
        T = random_transform()
        assert T.inv * (T * pg) == pg


def test_parallel_project_point_relations():
    p = vc.to_vec((3, 5, 7))
    for pg in _par_geoms():
        assert pg.project_point(pg.det_pos) == pytest.approx(np.zeros((pg.num_angles, 2)))
        with pytest.warns(UserWarning):
            moved = ts.translate(pg.ray_dir) * pg  # along the rays: same projection
        assert pg.project_point(p) == pytest.approx(moved.project_point(p))
        with pytest.warns(UserWarning):
            moved = ts.translate(pg.det_normal) * pg
        assert pg.project_point(p) == pytest.approx(moved.project_point(p))
        with pytest.warns(UserWarning):
            moved = ts.translate(pg.det_v + pg.det_u) * pg  # one pixel along v and u
        assert pg.project_point(p) - moved.project_point(p) == pytest.approx(
            np.ones((pg.num_angles, 2)))


def test_cone_project_point_of_detector_centre():
    for pg in _cone_geoms():
        assert pg.project_point(pg.det_pos) == pytest.approx(np.zeros((pg.num_angles, 2)),
                                                            abs=1e-9)


# -------------------------------------------------------------------- volumes
def test_volume_operations():
    vg = ts.volume()
    t = (5, 5, 5)
    assert vg in vg and vg in vg.scale(2)
    assert vg not in vg.translate(t) and vg not in vg.scale(0.5)
    assert vg.translate(t) in vg.translate(t).scale(2)
    assert vg.reshape(100) == vg.reshape((100,) * 3)
    v3 = ts.volume(shape=(3, 5, 7))
    assert np.allclose(v3.to_vec().size, v3.size)
    v10 = ts.volume(shape=10, size=10, pos=0)
    assert v10.with_voxel_size(1.0) == v10
    assert v10.with_voxel_size(2.0) == ts.volume(shape=5, size=10, pos=0)
    assert v10.with_voxel_size(3.0) == v10.with_voxel_size((3.0, 3.0, 3.0))


# ---------------------------------------------------------------- concatenate
def test_concatenate_transforms():
    t = random_transform()
    tt = ts.concatenate([t, t])
    assert tt.num_steps == 2 * t.num_steps and tt[: t.num_steps] == t


@pytest.mark.parametrize("make", [random_cone, random_cone_vec, random_parallel,
                                  random_parallel_vec, random_volume, random_volume_vec])
def test_concatenate_geometries(make):
    g = make()
    gg = ts.concatenate([g, g])
    assert gg.num_steps == 2 * g.num_steps
    assert gg[: g.num_steps] == g.to_vec() and gg[g.num_steps:] == g.to_vec()


def test_concatenate_errors():
    with pytest.raises(TypeError):
        ts.concatenate(ts.volume())  # not a sequence
    with pytest.raises(TypeError):
        ts.concatenate([ts.volume(), ts.parallel()])
    with pytest.raises(ValueError):
        ts.concatenate([])
    with pytest.raises(ValueError):
        ts.concatenate([ts.parallel(shape=3), ts.parallel(shape=4)])
    with pytest.raises(ValueError):
        ts.concatenate([ts.volume(shape=3), ts.volume(shape=4)])


def test_concatenated_scans_project_as_one():
    """Two half scans joined by concatenate describe the same rays as the full
    scan: their vectors match the full geometry's, angle for angle."""
    full = ts.cone(angles=8, shape=(4, 6), size=(1, 1.5), src_orig_dist=3, src_det_dist=5)
    joined = ts.concatenate([full[:4], full[4:]])
    v = full.to_vec()
    for name in ("src_pos", "det_pos", "det_v", "det_u"):
        assert getattr(joined, name) == pytest.approx(getattr(v, name))


def test_det_vec_astra_round_trip_and_conversion_module():
    """The detector-only geometry converts to tomosipo's ``det_vec`` pseudo-type
    and back, through ``ts.from_astra`` and the ``ts.geometry.conversion`` name."""
    from tomosipo_gb300.geometry import random_det_vec

    for _ in range(5):
        g = random_det_vec()
        d = g.to_astra()
        assert d["type"] == "det_vec" and d["Vectors"].shape == (g.num_angles, 12)
        assert ts.from_astra(d) == g
        assert ts.geometry.conversion.from_astra_projection_geometry(d) == g
    with pytest.raises(ValueError):
        ts.geometry.conversion.from_astra_projection_geometry({"type": "fanflat"})


# ------------------------------------------------------- detector-only vectors
def _det_vecs():
    from tomosipo_gb300.geometry import random_det_vec

    np.random.seed(11)
    return [ts.geometry.det_vec(shape=(4, 6), det_pos=np.zeros((8, 3)), det_v=(1, 0, 0),
                                det_u=(0, 0, 1))] + [random_det_vec() for _ in range(4)]


def test_det_vec_slicing_bins_the_detector():
    for pg in _det_vecs():
        assert pg == pg[:] == pg[:, :] == pg[:, :, :]
        assert pg[1::2].num_angles == pg.num_angles // 2
        if pg.num_angles % 2 or pg.det_shape[0] % 2 or pg.det_shape[1] % 2:
            continue
        assert pg[:, ::2].det_v == pytest.approx(2 * pg.det_v)
        assert pg[:, :, ::2].det_u == pytest.approx(2 * pg.det_u)
        assert pg[:, ::2].det_pos != pytest.approx(pg[:, 1::2].det_pos)
        assert pg[:, ::2, :].det_sizes == pytest.approx(pg[:, 1::2, :].det_sizes)
        assert pg[:, :, ::2].det_sizes == pytest.approx(pg[:, :, 1::2].det_sizes)


def test_det_vec_properties_and_transforms():
    for pg in _det_vecs():
        assert pg == pg.to_vec()
        assert pg.det_pos == pytest.approx(pg.to_vol().pos)
        with pytest.raises(NotImplementedError):
            pg.src_pos
        with pytest.raises(NotImplementedError):
            pg.ray_dir
        with pytest.raises(NotImplementedError):
            pg.project_point((0, 0, 0))
        assert pg.corners.shape == (pg.num_angles, 4, 3)
        assert pg.lower_left_corner == pytest.approx(pg.corners[:, 0, :])
        T1, T2 = random_transform(), random_transform()
        assert (T1 * T2) * pg == T1 * (T2 * pg)
        assert transform.identity() * pg == pg
        if pg.det_shape[0] % 2 == 0 and pg.det_shape[1] % 2 == 0:
            assert pg.rescale_det(2).det_v == pytest.approx(2 * pg.det_v)
    unit = ts.geometry.det_vec(shape=1, det_pos=(0, 0, 0), det_v=(1, 0, 0), det_u=(0, 0, 1))
    assert unit.det_normal == pytest.approx(np.array([(0, 1, 0)]))


# ------------------------------------------------------------- volume vectors
def test_volume_vec_init_and_repr():
    z, y, x = (1, 0, 0), (0, 1, 0), (0, 0, 1)
    ob = ts.volume_vec(shape=1, pos=0, w=z, v=y, u=x)
    assert ob == ts.volume_vec(shape=1, pos=0, w=z, v=y)
    assert ob == ts.volume_vec(shape=1, pos=0, w=[z], v=y)
    assert ob == ts.volume_vec(shape=(1, 1, 1), pos=[(0, 0, 0)], w=z, v=y, u=x)
    n = 11
    for bad in (dict(pos=[(0, 0, 0)] * 3, w=[z] * n, v=[y] * n, u=[x] * n),
                dict(pos=[(0, 0, 0)] * n, w=[z] * 3, v=[y] * n, u=[x] * n),
                dict(pos=[(0, 0, 0)] * n, w=[z] * n, v=[y] * 3, u=[x] * n),
                dict(pos=[(0, 0, 0)] * n, w=[z] * n, v=[y] * n, u=[x] * 3)):
        with pytest.raises(ValueError):
            ts.volume_vec(shape=1, **bad)
    unit_box = ts.volume_vec(shape=1, pos=(0, 0, 0))
    expected = """ts.volume_vec(
    shape=(1, 1, 1),
    pos=array([[0., 0., 0.]]),
    w=array([[1., 0., 0.]]),
    v=array([[0., 1., 0.]]),
    u=array([[0., 0., 1.]]),
)"""
    assert repr(unit_box) == expected
    with np.printoptions(legacy="1.13"):
        assert repr(unit_box) == expected
    for vg in (random_volume_vec(), ts.volume(shape=(3, 5, 7)).to_vec()):
        assert eval(repr(vg), dict(ts=ts, array=np.array)) == vg


def test_volume_vec_indexing_and_transforms():
    vg = random_volume_vec()
    assert vg[0] == vg[:1] == vg[-1] == vg[:] == vg
    assert ts.concatenate([vg, vg])[0] == vg and ts.concatenate([vg, vg])[1] == vg
    assert vg[np.ones(len(vg)) == 1] == vg
    assert vg[np.arange(len(vg)) % 2 == 0] == vg[0::2]
    assert ts.volume_vec(shape=3)[:, 1, 1, 1] == ts.volume_vec(shape=1)
    T = random_transform()
    assert T * vg[:, 1, 2, 3] == (T * vg)[:, 1, 2, 3]
    assert T * vg[:, :1, :2, :3] == (T * vg)[:, :1, :2, :3]
    assert T * vg[:, 1:, 2:, 3:] == (T * vg)[:, 1:, 2:, 3:]
    with pytest.raises(ValueError):
        vg[1, 2, 3, 4, 5]
    Tt = ts.translate(np.random.normal(size=3))
    assert (Tt * vg).w == pytest.approx(vg.w) and (Tt * vg).u == pytest.approx(vg.u)
    assert (Tt * vg).size == vg.size and (Tt * vg).voxel_size == vg.voxel_size
    S = ts.scale(abs(np.random.normal(size=(3, 3))))  # different scaling at each step and axis
    with pytest.raises(ValueError):
        (S * random_volume().to_vec()).size


def test_volume_vec_corners():
    zero, z, y, x = (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)
    n = 11
    vg = ts.volume_vec(shape=1, pos=[zero] * n, w=[z] * n, v=[y] * n, u=[x] * n)
    assert vg.corners.shape == (n, 8, 3)
    assert np.allclose(ts.volume_vec(shape=1, pos=0).lower_left_corner, [(-0.5,) * 3])
    assert np.allclose(ts.volume_vec(shape=1, pos=(0.5,) * 3).lower_left_corner, [(0,) * 3])
    frame = dict(w=(2, 3, 5), v=(7, 11, 13), u=(17, 19, 23))
    small = ts.volume_vec(shape=(1, 2, 3), pos=zero, **frame)
    big = ts.volume_vec(shape=(2, 4, 6), pos=zero, **frame)
    assert np.abs(small.corners * 2.0 - big.corners).sum() == pytest.approx(0.0)
    moved = ts.volume_vec(shape=(1, 2, 3), pos=(5, 7, 11), w=z, v=y, u=x)
    base = ts.volume_vec(shape=(1, 2, 3), pos=zero, w=z, v=y, u=x)
    assert np.abs((moved.corners - base.corners) - (5, 7, 11)).sum() == pytest.approx(0.0)


# ---------------------------------------------------------- vector geometries
def test_parallel_vec_init_validation_repr_and_equality():
    vecs = np.arange(30).reshape((10, 3))
    kw = dict(ray_dir=vecs, det_pos=vecs, det_v=vecs, det_u=vecs)
    assert ts.parallel_vec(shape=1, **kw).det_shape == (1, 1)
    assert ts.parallel_vec(shape=(3, 5), **kw).det_shape == (3, 5)
    with pytest.raises(TypeError):
        ts.parallel_vec(1, **kw)  # shape is keyword-only
    with pytest.raises(TypeError):
        ts.parallel_vec(shape=0, **kw)
    with pytest.raises(TypeError):
        two = np.random.normal(size=(10, 2))
        ts.parallel_vec(shape=1, ray_dir=two, det_pos=two, det_v=two, det_u=two)
    with pytest.raises(ValueError):
        ts.parallel_vec(shape=1, ray_dir=np.random.normal(size=(10, 3)),
                        det_pos=np.random.normal(size=(11, 3)),
                        det_v=np.random.normal(size=(12, 3)), det_u=np.random.normal(size=(13, 3)))
    x = [[1, 2, 3], [4, 5, 6]]
    pg = ts.parallel_vec(shape=10, ray_dir=x, det_pos=x, det_v=x, det_u=x)
    expected = """ts.parallel_vec(
    shape=(10, 10),
    ray_dir=array([[1., 2., 3.],
       [4., 5., 6.]]),
    det_pos=array([[1., 2., 3.],
       [4., 5., 6.]]),
    det_v=array([[1., 2., 3.],
       [4., 5., 6.]]),
    det_u=array([[1., 2., 3.],
       [4., 5., 6.]]),
)"""
    assert repr(pg) == expected
    with np.printoptions(legacy="1.13"):
        assert repr(pg) == expected
    r = random_parallel()
    assert eval(repr(r), dict(ts=ts, array=np.array)) == r
    z = np.array([(0, 0, 0)])
    pg = ts.parallel_vec(shape=10, ray_dir=z, det_pos=z, det_v=z, det_u=z)
    unequal = [ts.parallel_vec(shape=9, ray_dir=z, det_pos=z, det_v=z, det_u=z),
               ts.parallel_vec(shape=10, ray_dir=z + 1, det_pos=z, det_v=z, det_u=z),
               ts.parallel_vec(shape=10, ray_dir=z, det_pos=z + 1, det_v=z, det_u=z),
               ts.parallel_vec(shape=10, ray_dir=z, det_pos=z, det_v=z + 1, det_u=z),
               ts.parallel_vec(shape=10, ray_dir=z, det_pos=z, det_v=z, det_u=z + 1),
               ts.cone(size=np.sqrt(2), cone_angle=0.5, angles=2),
               ts.cone(size=np.sqrt(2), cone_angle=0.5).to_vec(), ts.volume()]
    assert pg == pg
    for u in unequal:
        assert u != pg and pg != u


@pytest.mark.parametrize("make", [random_parallel_vec, random_cone_vec])
def test_vector_geometry_slicing(make):
    for _ in range(4):
        pg = make()
        assert pg == pg[:] == pg[:, :] == pg[:, :, :]
        assert pg[np.ones(pg.num_angles) == 1] == pg
        assert pg[np.arange(pg.num_angles) % 2 == 0] == pg[0::2]
        assert pg[1::2].num_angles == pg.num_angles // 2
        assert pg[1:9:2].det_pos == pytest.approx(pg.det_pos[1:9:2, :])
        assert pg[-1].det_pos == pytest.approx(pg.det_pos[-1:, :])
        if pg.num_angles % 2 or pg.det_shape[0] % 2 or pg.det_shape[1] % 2:
            continue
        assert pg[:, ::2].det_v == pytest.approx(2 * pg.det_v)
        assert pg[:, :, ::2].det_u == pytest.approx(2 * pg.det_u)
        assert pg[:, ::2].det_pos != pytest.approx(pg[:, 1::2].det_pos)
        assert pg[:, ::2, :].det_sizes == pytest.approx(pg[:, 1::2, :].det_sizes)


# ------------------------------------------------------------- plain volumes
def test_volume_pos_size_extent():
    from tomosipo_gb300.geometry.volume import _extent_to_pos_size, _pos_size_to_extent

    for _ in range(10):
        pos, size = np.random.normal(size=3), np.square(np.random.normal(size=3))
        p2, s2 = _extent_to_pos_size(_pos_size_to_extent(pos, size))
        assert np.allclose(p2, pos) and np.allclose(s2, size)
    assert ts.geometry.is_volume(ts.volume()) and ts.geometry.is_volume(ts.volume().to_vec())
    assert not ts.geometry.is_volume(ts.cone(cone_angle=0.5)) and not ts.geometry.is_volume(None)
    assert ts.volume().shape == (1, 1, 1) and ts.volume(shape=(3, 4, 5)).shape == (3, 4, 5)
    extent = ((0, 1), (3, 4), (5, 6))
    assert ts.volume(extent=extent).extent == extent
    assert ts.volume(pos=(0.5, 0.5, 0.5), size=1).extent == ((0, 1),) * 3
    # pos and size, or extent, not both
    for kw in (dict(pos=0, size=1, extent=extent), dict(pos=0, extent=extent),
               dict(size=1, extent=extent)):
        with pytest.raises(ValueError):
            ts.volume(**kw)
    for kw in (dict(pos=0, size=1), dict(pos=0), dict(size=1), dict(extent=extent), dict()):
        ts.volume(**kw)
    for bad in ((1, 0), 3):
        with pytest.raises(TypeError):
            ts.volume(extent=bad)
    with pytest.raises(TypeError):
        ts.volume(shape=0)


def test_volume_equality_repr_and_indexing():
    vg = ts.volume()
    for u in (ts.volume(shape=10), ts.volume(shape=(10, 9, 8)), ts.cone(cone_angle=0.5)):
        assert vg != u
    box = ts.volume(shape=(1, 2, 3), pos=(4, 5, 6), size=(7, 8, 9))
    assert repr(box) == """ts.volume(
    shape=(1, 2, 3),
    pos=(4.0, 5.0, 6.0),
    size=(7.0, 8.0, 9.0),
)"""
    r = random_volume()
    assert eval(repr(r), dict(ts=ts)) == r
    assert len(ts.volume()) == 1
    moved = ts.volume().scale((1, 2, 3)).translate((10, 20, 30))
    assert ts.from_astra(moved.to_astra()) == moved
    vg = ts.volume(shape=(3, 4, 5), extent=((11, 13), (17, 19), (23, 29)))
    assert vg == vg[:, :, :] == vg[:, :] == vg[:]
    assert vg[0, 0, 0] == vg[:1, :1, :1] and vg[0] == vg[0, :, :] and vg[-1] == vg[2]
    assert vg[::3, ::4, ::5].shape == (1, 1, 1)
    assert np.allclose(vg[0, 1, 2].size, np.array(vg.size) / vg.shape)  # voxel size kept
    assert np.allclose(vg.size[1], vg[:, ::2, :].size[1])
    assert vg.shape[1] == 2 * vg[:, ::2].shape[1]
    assert np.allclose(vg[:, ::2, :].size, vg[:, 1::2, :].size)


# ------------------------------------------------- constructors, repr, equality
def test_cone_constructor_rules():
    with pytest.raises(TypeError):
        ts.cone(angles=1, shape=None, cone_angle=1)
    with pytest.raises(TypeError):
        ts.cone(angles=None, shape=1, cone_angle=1)
    kw = dict(angles=1, shape=1, size=1)
    # cone_angle alone, or distances without it; not both, not neither
    for bad in (dict(cone_angle=1, src_orig_dist=1, src_det_dist=1),
                dict(cone_angle=1, src_orig_dist=1), dict(cone_angle=1, src_det_dist=1), dict()):
        with pytest.raises(ValueError):
            ts.cone(**kw, **bad)
    for ok in (dict(cone_angle=1), dict(src_orig_dist=1, src_det_dist=1),
               dict(src_orig_dist=1), dict(src_det_dist=1)):
        ts.cone(**kw, **ok)
    assert ts.cone(shape=2, cone_angle=1).det_size == (2, 2)  # size defaults to shape
    assert ts.cone(shape=2, size=1, cone_angle=1).det_size == (1, 1)
    assert isinstance(ts.cone(cone_angle=1), ts.geometry.ProjectionGeometry)
    assert ts.cone(angles=np.linspace(0, 1, 100), cone_angle=1).num_angles == 100
    with pytest.raises(TypeError):
        ts.cone(size=np.sqrt(2), cone_angle=0.5, angles=[])


def test_parallel_constructor_rules():
    assert ts.parallel(angles=1, shape=1).det_shape == (1, 1)
    assert ts.parallel(angles=1, size=1).det_sizes == pytest.approx(np.ones((1, 2)))
    assert ts.parallel(shape=(2, 3)).det_size == (2, 3) and ts.parallel().det_shape == (1, 1)
    assert ts.parallel(angles=10) == ts.parallel(angles=np.linspace(0, np.pi, 10, endpoint=False))
    for bad in (dict(shape=0), dict(angles=0), dict(angles=np.ones((1, 1)))):
        with pytest.raises(TypeError):
            ts.parallel(**bad)


def test_cone_and_parallel_repr_and_equality():
    pg = ts.cone(angles=10, shape=11, size=1, src_orig_dist=5, src_det_dist=6)
    expected = """ts.cone(
    angles=10,
    shape=(11, 11),
    size=(1.0, 1.0),
    src_orig_dist=5.0,
    src_det_dist=6.0,
)"""
    assert repr(pg) == expected
    with np.printoptions(legacy="1.13"):
        assert repr(pg) == expected
    pg = ts.parallel(angles=10, shape=11, size=1)
    assert repr(pg) == """ts.parallel(
    angles=10,
    shape=(11, 11),
    size=(1.0, 1.0),
)"""
    for make in (random_cone, random_parallel):
        g = make()
        assert eval(repr(g), dict(ts=ts, array=np.array)) == g
    cg = ts.cone(size=np.sqrt(2), cone_angle=0.5)
    for u in (ts.cone(size=5, cone_angle=0.5), ts.cone(angles=2, size=np.sqrt(2), cone_angle=0.5),
              ts.cone(shape=2, size=np.sqrt(2), cone_angle=0.5),
              ts.cone(size=np.sqrt(2), src_orig_dist=50), ts.cone(size=np.sqrt(2), src_det_dist=50),
              ts.volume()):
        assert cg != u
    par = ts.parallel()
    for u in (ts.parallel(angles=2), ts.parallel(size=5), ts.parallel(shape=3), ts.volume()):
        assert u != par and par != u


def test_cone_vec_validation_repr_and_equality():
    vecs = np.arange(30).reshape((10, 3))
    kw = dict(src_pos=vecs, det_pos=vecs, det_v=vecs, det_u=vecs)
    repr(ts.cone_vec(shape=1, **kw))
    with pytest.raises(TypeError):
        ts.cone_vec(0, **kw)  # shape is keyword-only
    with pytest.raises(TypeError):
        ts.cone_vec(shape=0, **kw)
    two = np.arange(20).reshape((10, 2))
    with pytest.raises(TypeError):
        ts.cone_vec(shape=1, src_pos=two, det_pos=two, det_v=two, det_u=two)
    with pytest.raises(ValueError):
        ts.cone_vec(shape=1, src_pos=np.random.normal(size=(10, 3)),
                    det_pos=np.random.normal(size=(11, 3)),
                    det_v=np.random.normal(size=(12, 3)), det_u=np.random.normal(size=(13, 3)))
    x = [[1, 2, 3], [4, 5, 6]]
    expected = """ts.cone_vec(
    shape=(10, 10),
    src_pos=array([[1., 2., 3.],
       [4., 5., 6.]]),
    det_pos=array([[1., 2., 3.],
       [4., 5., 6.]]),
    det_v=array([[1., 2., 3.],
       [4., 5., 6.]]),
    det_u=array([[1., 2., 3.],
       [4., 5., 6.]]),
)"""
    pg = ts.cone_vec(shape=10, src_pos=x, det_pos=x, det_v=x, det_u=x)
    assert repr(pg) == expected
    with np.printoptions(legacy="1.13"):
        assert repr(pg) == expected
    r = random_cone_vec()
    assert eval(repr(r), dict(ts=ts, array=np.array)) == r
    z = np.array([(0, 0, 0)])
    pg = ts.cone_vec(shape=10, src_pos=z, det_pos=z, det_v=z, det_u=z)
    for u in (ts.cone_vec(shape=9, src_pos=z, det_pos=z, det_v=z, det_u=z),
              ts.cone_vec(shape=10, src_pos=z + 1, det_pos=z, det_v=z, det_u=z),
              ts.cone_vec(shape=10, src_pos=z, det_pos=z + 1, det_v=z, det_u=z),
              ts.cone_vec(shape=10, src_pos=z, det_pos=z, det_v=z + 1, det_u=z),
              ts.cone_vec(shape=10, src_pos=z, det_pos=z, det_v=z, det_u=z + 1),
              ts.cone(angles=2, cone_angle=0.5), ts.volume()):
        assert pg != u
    big = ts.cone(angles=10, shape=100, size=np.sqrt(2), cone_angle=0.5).to_vec()
    assert 10 * big[::10].num_angles == big.num_angles
    assert np.abs(big[:, ::2].det_v - 2 * big.det_v).sum() == pytest.approx(0.0, abs=1e-7)
    assert np.abs(big[:, :, ::2].det_pos - big[:, :, 1::2].det_pos).sum() > 1e-7


def test_projection_geometry_interface():
    """The common interface every projection geometry answers
    (tomosipo's ``tests/geometry/test_base_projection.py``)."""
    from tomosipo_gb300.geometry import ProjectionGeometry, is_projection, random_det_vec

    geoms = [ts.cone(size=np.sqrt(2), cone_angle=0.5), ts.cone(size=np.sqrt(2), cone_angle=0.5).to_vec(),
             ts.cone(angles=10, shape=(5, 3), cone_angle=0.5),
             ts.cone(size=np.sqrt(2), cone_angle=0.5, angles=11, shape=(10, 10)).to_vec(),
             random_det_vec(), random_parallel_vec(), random_parallel()]
    assert not is_projection(ts.volume()) and not is_projection(None)
    assert ProjectionGeometry().det_shape == (1, 1)
    with pytest.raises(TypeError):
        ProjectionGeometry(0)
    for pg in geoms:
        assert is_projection(pg) and pg == pg
        repr(pg)
        fixed = ts.from_astra(pg.to_astra())
        assert fixed == ts.from_astra(fixed.to_astra())
        assert pg.to_vec() == pg.to_vec().to_vec()
        assert len(pg) == pg.num_angles
        if pg.is_vec:
            with pytest.raises(NotImplementedError):
                pg.angles
        else:
            assert len(pg.angles) == pg.num_angles
        if pg.is_cone:
            assert pg.src_pos.shape == (pg.num_angles, 3)
        if pg.is_parallel:
            assert pg.ray_dir.shape == (pg.num_angles, 3)
        for name in ("det_pos", "det_v", "det_u"):
            assert getattr(pg, name).shape == (pg.num_angles, 3)
        assert vc.cross_product(pg.det_u, pg.det_v) == pytest.approx(pg.det_normal)
        if pg.is_vec and pg.num_angles > 1:
            # a detector whose size changes from angle to angle has no single size
            S = ts.scale(np.abs(np.random.normal(size=(pg.num_angles, 3))) + 0.5)
            with pytest.raises(ValueError):
                (S * pg).det_size
        else:
            assert len(pg.det_size) == 2
        assert pg.det_sizes.shape == (pg.num_angles, 2)
        assert pg.corners.shape == (pg.num_angles, 4, 3)
        assert pg.reshape(1).det_shape == (1, 1)
        if pg.is_parallel or pg.is_cone:
            pg.project_point((0, 0, 0))


def test_operator_needs_a_ray_geometry():
    """A volume or a detector alone defines no rays: a TypeError at creation
    (host only; the native projector is made on first use)."""
    from tomosipo_gb300.geometry import random_det_vec

    vg = ts.volume(shape=8)
    for pg in (random_det_vec(), ts.volume(shape=8)):
        with pytest.raises(TypeError, match="parallel or cone"):
            ts.operator(vg, pg)
    with pytest.raises(TypeError):
        ts.operator(ts.parallel(angles=3), vg)  # arguments swapped
    for pg in (ts.parallel(angles=3), ts.cone(angles=3, cone_angle=0.5)):
        A = ts.operator(vg, pg)
        assert A.domain_shape == (8, 8, 8) and A.range_shape == (1, 3, 1)
        assert A.T.T is A and A.domain == vg and A.range == pg
