"""Geometry conventions, pinned by the reference's own docs and tests.

Each expected value below is quoted from the tomosipo file cited beside it.
"""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300.geometry import random_transform, random_volume_vec


def test_parallel_to_vec_matches_doc():
    # doc/topics/geometries.rst:364-410 (pg = ts.parallel(angles=3, shape=(10, 15), size=(1, 1.5)))
    pg = ts.parallel(angles=3, shape=(10, 15), size=(1, 1.5))
    assert np.allclose(pg.det_pos, 0)
    assert np.allclose(pg.det_v, [[0.1, 0, 0]] * 3)
    assert np.allclose(pg.det_u, [[0, 0, 0.1], [0, 0.08660254, 0.05], [0, 0.08660254, -0.05]])
    assert np.allclose(pg.ray_dir, [[0, -1, 0], [0, -0.5, 0.8660254], [0, 0.5, 0.8660254]])
    assert np.allclose(pg.det_normal, [[0, 0.01, 0], [0, 0.005, -0.00866025], [0, -0.005, -0.00866025]])
    assert np.allclose(
        pg.lower_left_corner,
        [[-0.5, 0, -0.75], [-0.5, -0.64951905, -0.375], [-0.5, -0.64951905, 0.375]],
    )
    assert np.allclose(
        pg.corners[1],
        [[-0.5, -0.64951905, -0.375], [0.5, -0.64951905, -0.375],
         [-0.5, 0.64951905, 0.375], [0.5, 0.64951905, 0.375]],
    )


def test_angle_defaults():
    # parallel: half arc (tomosipo/geometry/parallel.py:86-88); cone: full arc (cone.py:164-166)
    assert np.allclose(ts.parallel(angles=4).angles, np.linspace(0, np.pi, 4, endpoint=False))
    assert np.allclose(ts.cone(angles=4, cone_angle=0.5).angles, np.linspace(0, 2 * np.pi, 4, endpoint=False))


def test_cone_project_point_detector_spacing():
    # tests/geometry/test_cone_vec.py:143-173
    pg = ts.cone(angles=1, shape=(10, 40), size=(30, 80), src_orig_dist=10, src_det_dist=10).to_vec()
    assert np.abs(pg.project_point((0, 0, 0))).sum() == pytest.approx(0, abs=1e-7)
    assert np.abs(pg.project_point((3.0, 0, 0)) - [1.0, 0.0]).sum() == pytest.approx(0, abs=1e-7)
    assert np.abs(pg.project_point((0, 0, 2.0)) - [0.0, 1.0]).sum() == pytest.approx(0, abs=1e-7)
    pg = ts.cone(angles=1, shape=(100, 400), size=(30, 80), src_orig_dist=10, src_det_dist=10).to_vec()
    assert np.abs(pg.project_point((0.3, 0, 0)) - [1.0, 0.0]).sum() == pytest.approx(0, abs=1e-7)
    assert np.abs(pg.project_point((0, 0, 0.2)) - [0.0, 1.0]).sum() == pytest.approx(0, abs=1e-7)


def test_cone_src_pos_scales_with_distance():
    # tests/geometry/test_cone_vec.py:196-201
    pg1 = ts.cone(size=np.sqrt(2), src_orig_dist=1, src_det_dist=1).to_vec()
    pg2 = ts.cone(size=np.sqrt(2), src_orig_dist=2, src_det_dist=2).to_vec()
    assert np.all(abs(pg1.src_pos * 2 - pg2.src_pos) < ts.epsilon)
    assert np.allclose(np.linalg.norm(pg2.src_pos, axis=1), 2)


def test_cone_angle_places_detector_at_origin():
    # tomosipo/geometry/cone.py:82-85: src_orig_dist = src_det_dist = height / cone_angle
    pg = ts.cone(angles=5, shape=(10, 20), size=(2.0, 3.0), cone_angle=0.5)
    assert pg.src_orig_dist == pg.src_det_dist == 4.0
    assert np.allclose(pg.to_vec().det_pos, 0)


def test_det_sizes_reshape():
    # tests/geometry/test_cone_vec.py:176-186
    pg = ts.cone(angles=5, size=(1, 1), cone_angle=1 / 2).to_vec()
    assert abs(np.array((1, 1)) - pg.det_sizes).sum() < ts.epsilon
    for shape in [(3, 7), (50, 2), (99, 99)]:
        pg2 = pg.reshape(shape)
        assert pg2.det_shape == shape
        assert np.abs(pg2.det_sizes - pg.det_sizes).sum() == pytest.approx(0, abs=1e-7)


def test_volume_indexing_doctest():
    # doc/topics/geometries.rst:68-91
    vg = ts.volume(shape=3)
    assert vg[0, 0, 0] == ts.volume(shape=1, pos=(-1, -1, -1), size=1)
    assert vg[2, 0, 0] == ts.volume(shape=1, pos=(1, -1, -1), size=1)
    assert vg[2, 2, 2] == ts.volume(shape=1, pos=(1, 1, 1), size=1)
    vg = ts.volume(shape=128)
    assert vg[64, :, :] == vg[64]


def test_volume_voxel_centres():
    vg = ts.volume(shape=(4, 5, 6), pos=(1, 2, 3), size=(2, 3, 4))
    assert vg.voxel_size == (0.5, 0.6, 4 / 6)
    llc = vg.lower_left_corner[0]
    assert np.allclose(llc, np.array((1, 2, 3)) - np.array((2, 3, 4)) / 2)
    assert vg.extent == ((0.0, 2.0), (0.5, 3.5), (1.0, 5.0))
    assert ts.volume(shape=4, extent=((0, 2), (0.5, 3.5), (1, 5))).size == (2.0, 3.0, 4.0)


def test_transform_doctests():
    # tomosipo/geometry/transform.py doctests (translate, scale, to/from_perspective)
    assert np.allclose(ts.translate((1, 2, 3)).matrix[0, :3, 3], (1, 2, 3))
    assert np.allclose(ts.translate((1, 1, 1), alpha=[2, 3]).matrix[:, 0, 3], (2, 3))
    assert np.allclose(ts.scale((2, 2, 2), pos=(3, 4, 5)).matrix[0, :3, 3], (-3, -4, -5))
    assert np.allclose(ts.scale(1, alpha=[2, 3]).matrix[:, 0, 0], (2, 3))
    P = ts.from_perspective(pos=(1, 2, 3), w=(2, 0, 0), v=(0, 2, 0), u=(0, 0, 2), ignore_scale=False)
    assert np.allclose(P.matrix[0], [[0.5, 0, 0, -0.5], [0, 0.5, 0, -1], [0, 0, 0.5, -1.5], [0, 0, 0, 1]])
    with pytest.raises(ValueError):
        ts.translate((1, 0, 0), alpha=[0, 1]) * ts.translate((1, 0, 0), alpha=[0, 1, 2])


def test_rotate_right_handed():
    # right-handed rotation about z maps x to y
    R = ts.rotate(pos=0, axis=(1, 0, 0), angles=np.pi / 2)
    assert np.allclose(R.transform_point((0, 0, 1)), (0, 1, 0))
    L = ts.rotate(pos=0, axis=(1, 0, 0), angles=np.pi / 2, right_handed=False)
    assert np.allclose(L.transform_point((0, 0, 1)), (0, -1, 0))


def test_transform_inverse_and_geometry_roundtrip():
    rng_state = np.random.get_state()
    np.random.seed(3)
    try:
        for _ in range(5):
            T = random_transform()
            vg = random_volume_vec()
            assert T.inv * (T * vg) == vg
            pg = ts.geometry.random_cone_vec()
            assert T.inv * (T * pg) == pg
    finally:
        np.random.set_state(rng_state)


@pytest.mark.parametrize(
    "pg",
    [
        ts.parallel(angles=5, shape=(3, 4), size=(1, 2)),
        ts.cone(angles=5, shape=(3, 4), size=(1, 2), src_orig_dist=3, src_det_dist=5),
        ts.parallel(angles=5, shape=(3, 4), size=(1, 2)).to_vec(),
        ts.cone(angles=5, shape=(3, 4), size=(1, 2), src_orig_dist=3, src_det_dist=5).to_vec(),
    ],
)
def test_astra_roundtrip(pg):
    # tests/test_astra.py:24-41 (ts.to_astra / ts.from_astra)
    assert ts.from_astra(ts.to_astra(pg)) == pg
    with pytest.raises(TypeError):
        ts.from_astra(pg)  # a geometry is not an ASTRA dict
    with pytest.raises(TypeError):
        ts.to_astra(ts.to_astra(pg))  # nor is a dict a geometry


def test_volume_astra_roundtrip():
    vg = ts.volume(shape=(3, 4, 5), pos=(0.1, 0.2, 0.3), size=(1, 2, 3))
    assert ts.from_astra(ts.to_astra(vg)) == vg


def test_geometry_shape():
    # tomosipo/links/base.py:21-31
    from tomosipo_gb300.links import geometry_shape

    assert geometry_shape(ts.volume(shape=(3, 4, 5))) == (3, 4, 5)
    assert geometry_shape(ts.parallel(angles=7, shape=(2, 9))) == (2, 7, 9)


def test_slicing_bins_pixels():
    # tomosipo/utils.py:45-119: strided slices keep the first pixel centre, scale the pixel
    pg = ts.parallel(shape=10).to_vec()
    assert pg[:, ::2, ::2].det_shape == (5, 5)
    assert ts.parallel(angles=10)[0::2].num_angles == 5
    assert ts.cone(angles=10, cone_angle=1 / 2).to_vec()[0::2].num_angles == 5


def test_volume_vec_with_operator_normalisation():
    # tomosipo/Operator.py:11-60: vec volume -> axis-aligned volume at the origin
    from tomosipo_gb300.Operator import to_astra_compatible_operator_geometry

    R = ts.rotate(pos=0, axis=(1, 2, 3), angles=0.4)
    T = ts.translate((0.3, -0.2, 0.1))
    vg = ts.volume(shape=(8, 9, 10), size=(1, 1.5, 2))
    pg = ts.cone(angles=4, shape=(5, 6), size=3, src_orig_dist=5, src_det_dist=7).to_vec()
    vg2, pg2 = to_astra_compatible_operator_geometry(T * R * vg.to_vec(), T * R * pg)
    assert vg2 == ts.volume(shape=(8, 9, 10), size=(1, 1.5, 2))
    assert pg2 == pg


def test_hollow_box_phantom_mean():
    """tomosipo's only numeric known answer for the phantom
    (``tests/test_phantom.py:11-17``): a 100^3 hollow box has mean 0.208."""
    vd = ts.data(ts.volume(shape=100))
    ts.phantom.hollow_box(vd)
    assert vd.data.mean() == pytest.approx(0.208)


def test_reference_notebook_unit_cone_repr():
    """The reference's getting-started notebook prints the unit cone of the
    benchmark's geometry family and the default volume
    (``notebooks/00_getting_started_google_colab.ipynb`` cell 1): cone_angle
    0.5 with a sqrt(2) detector puts source and detector 2 sqrt(2) from the
    origin. The reprs here are the same text."""
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")) as f:
        pin = json.load(f)["colab_notebook_unit_cone_repr"]
    assert repr(ts.cone(angles=20, size=np.sqrt(2), cone_angle=0.5)) == pin["cone_repr"]
    assert repr(ts.volume()) == pin["volume_repr"]
