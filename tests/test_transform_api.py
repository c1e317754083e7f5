"""Transform algebra that tomosipo's ``tests/geometry/test_transform.py`` pins,
restated with seeded inputs: the group laws on geometries, vectors and
points; translate / scale / rotate composition and their ``alpha`` /
``pos`` / handedness parameters; reflections; and the perspective transforms
the operator uses to normalise volume-vector geometries. Host only.
"""
import itertools

import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300.geometry import random_volume_vec, transform

_rng = np.random.default_rng(50)
np.random.seed(50)
VGS = [ts.volume_vec(shape=1, pos=0), ts.volume_vec(shape=(3, 5, 7), pos=0),
       ts.volume_vec(shape=(3, 5, 7), pos=(0.1, -0.3, 4.5)), random_volume_vec()]
TRANSLATIONS = [ts.translate((0, 0, 0)), ts.translate(_rng.normal(0, 1, size=3))]
ROTATIONS = [
    ts.rotate(pos=0, axis=(1, 0, 0), angles=0),
    ts.rotate(pos=0, axis=(1, 0, 0), angles=1.0),
    ts.rotate(pos=0, axis=_rng.normal(size=3), angles=_rng.normal()),
    ts.rotate(pos=0, axis=_rng.normal(size=3), angles=_rng.normal(), right_handed=False),
]
REFLECTIONS = [ts.reflect(pos=0, axis=(1, 0, 0)), ts.reflect(pos=(1, 1, 1), axis=(1, 1, 1)),
               ts.reflect(pos=(0, 1, 1), axis=(0, -1, 1))]
SCALINGS = [ts.scale(1), ts.scale(abs(_rng.normal())), ts.scale(abs(_rng.normal(size=3)))]


@pytest.fixture(autouse=True)
def _seeded():
    np.random.seed(51)


@pytest.mark.parametrize(
    "vg, T, R, M, S",
    list(itertools.product(VGS[:2], TRANSLATIONS, ROTATIONS, REFLECTIONS[:2], SCALINGS)))
def test_group_laws_on_geometries(vg, T, R, M, S):
    I = transform.identity()
    assert I * vg == vg and I * S == S and I * T == T and I * R == R
    assert I * (S * T * R) == S * T * R
    assert S * (T * (R * (M * vg))) == (((S * T) * R) * M) * vg
    assert S * ((T * R) * M) == ((S * T) * R) * M
    for t in (I, S, T, R, M, S * T * R, S * T * R * M):
        assert I == t * t.inv and I == t.inv * t
    assert (T * S * R * M).inv == M.inv * R.inv * S.inv * T.inv


@pytest.mark.parametrize("T, R, S", list(itertools.product(TRANSLATIONS, ROTATIONS, SCALINGS)))
def test_group_laws_on_vectors_and_points(T, R, S):
    I = transform.identity()
    x = np.random.normal(size=(10, 3))
    for apply in ("transform_vec", "transform_point"):
        f = lambda t: getattr(t, apply)(x)  # noqa: E731
        assert f(I).shape == x.shape and np.allclose(f(I), x)
        assert np.allclose(f(I * S), f(S)) and np.allclose(f(I * T), f(T))
        assert np.allclose(f(S * (T * R)), f((S * T) * R))
        for t in (I, S, T, R, S * T * R):
            assert np.allclose(f(t * t.inv), x) and np.allclose(f(t.inv * t), x)
        assert np.allclose(f((T * S * R).inv), f(R.inv * S.inv * T.inv))


def test_equality_and_indexing():
    for T in TRANSLATIONS + ROTATIONS + SCALINGS:
        assert T == T
        assert T != ts.translate((0.1, 0.1, 0.1)) * T
        assert T != ts.scale(0.1) * T
        assert T != ts.rotate(pos=0, axis=(1, 0, 0), angles=1.0) * T
    for T in TRANSLATIONS:
        assert T[0] == T[:1] == T
        assert ts.concatenate([T, T])[0] == T and ts.concatenate([T, T])[1] == T
        with pytest.raises(TypeError):
            T[0, 0]


def test_translate():
    R = ts.rotate(pos=(2, 3, 5), axis=(7, 11, -13), angles=np.deg2rad(15))
    original = R * ts.volume_vec(shape=(3, 4, 5), pos=(2, 3, 5))
    t = np.array((3, 4, 5))
    assert ts.translate(t) * original == ts.volume_vec(
        shape=(3, 4, 5), pos=t + (2, 3, 5), w=original.w, v=original.v, u=original.u)
    for t1, t2 in np.random.normal(size=(5, 2, 3)):
        vg = random_volume_vec()
        T1, T2 = ts.translate(t1), ts.translate(t2)
        assert (T1 * T2) * vg == T1 * (T2 * vg)
        assert T1 * T2 == ts.translate(t1 + t2) == T2 * T1
    axis = np.array([1, 2, 3])
    T = ts.translate(axis)
    assert T * T == ts.translate(axis, alpha=2) and T * T * T == ts.translate(axis, alpha=3)
    assert ts.translate(axis, alpha=[2, 3]).num_steps == 2


def test_scale():
    unit = ts.volume_vec(shape=1, pos=0)
    s = abs(np.random.normal())
    assert ts.scale(s) * unit == ts.volume_vec(shape=1, pos=0, w=s * unit.w, v=s * unit.v,
                                               u=s * unit.u)
    s3 = abs(np.random.normal(size=3))
    assert ts.scale(s3) * unit == ts.volume_vec(shape=1, pos=0, w=s3[0] * unit.w,
                                                v=s3[1] * unit.v, u=s3[2] * unit.u)
    for s1, s2 in abs(np.random.normal(size=(5, 2, 3))):
        vg = random_volume_vec()
        assert (ts.scale(s1) * ts.scale(s2)) * vg == ts.scale(s1) * (ts.scale(s2) * vg)
        assert ts.scale(s1) * ts.scale(s2) == ts.scale(s1 * s2)
    for _ in range(5):
        vg = ts.translate(np.random.normal(size=3)) * random_volume_vec()
        assert np.allclose((ts.scale(3, pos=vg.pos) * vg).pos, vg.pos)  # about its centre
    s = np.array([1, 2, 3])
    assert ts.scale(2 * s) == ts.scale(s, alpha=2) and ts.scale(3 * s) == ts.scale(s, alpha=3)
    assert ts.scale(s, alpha=[2, 3]).num_steps == 2


def test_rotate():
    for p, axis in np.random.normal(size=(5, 2, 3)):
        a = 2 * np.pi * np.random.normal()
        R = ts.rotate(pos=p, axis=axis, angles=a, right_handed=True)
        assert R == ts.rotate(pos=p, axis=axis, angles=-a, right_handed=False)
        assert R == ts.rotate(pos=p, axis=-axis, angles=a, right_handed=False)
        assert R == ts.rotate(pos=p, axis=axis, angles=a + 2 * np.pi, right_handed=True)
        assert R == ts.rotate(pos=p, axis=2 * axis, angles=a, right_handed=True)
    for t1, t2 in np.random.normal(size=(5, 2)):
        vg = random_volume_vec()
        axis, pos = np.random.normal(size=3), np.random.normal(size=3)
        R1 = ts.rotate(pos=pos, axis=axis, angles=t1)
        R2 = ts.rotate(pos=pos, axis=axis, angles=t2)
        assert (R1 * R2) * vg == R1 * (R2 * vg)
        assert R1 * R2 == ts.rotate(pos=pos, axis=axis, angles=t1 + t2)
    for n in (2, 5):
        assert ts.rotate(pos=np.ones((n, 3)), axis=np.ones((n, 3)), angles=np.ones(n)).num_steps == n
        assert ts.rotate(pos=0, axis=np.ones((n, 3)), angles=np.ones(n)).num_steps == n
        assert ts.rotate(pos=np.ones((n, 3)), axis=(1, 0, 0), angles=np.ones(n)).num_steps == n
        assert ts.rotate(pos=np.ones((n, 3)), axis=np.ones((n, 3)), angles=0.15).num_steps == n


def test_reflect():
    vg = ts.volume(shape=1).to_vec()
    M = ts.reflect(pos=0, axis=(1, 0, 0))
    assert vg.size == (M * vg).size
    in_plane = np.array([[0.0, 1, 1], [0.0, 2, 0], [0.0, 0, 3]])
    assert np.allclose(in_plane, M.transform_point(in_plane))
    for p in np.array([[1.0, 1, 1], [-1.0, 2, 0], [3.0, 0, 3]]):
        assert not np.allclose(p, M.transform_point(p))
    for M in REFLECTIONS:
        assert transform.identity() == M * M and M.inv == M


def test_perspective():
    unit = ts.volume_vec(shape=1, pos=0)
    for t, p, axis in np.random.normal(size=(5, 3, 3)):
        R = ts.rotate(pos=p, axis=axis, angles=2 * np.pi * np.random.normal())
        box = (R * ts.translate(t)) * unit
        to_box = ts.to_perspective(vol=box)
        assert box == to_box * unit
        to_unit = ts.from_perspective(vol=box)
        assert unit == to_unit * box
        assert to_box * to_unit == transform.identity()
        assert to_box == ts.to_perspective(pos=box.pos, w=box.w, v=box.v, u=box.u)
    vg = ts.volume(shape=1, pos=0)
    large = ts.scale(2.0) * vg.to_vec()
    assert vg != ts.from_perspective(vol=large, ignore_scale=False) * vg.to_vec()
    assert vg.to_vec() == ts.from_perspective(vol=large, ignore_scale=True) * vg.to_vec()


def test_rotate_deprecated_keywords():
    with pytest.warns(DeprecationWarning):
        R = ts.rotate(pos=0, axis=(1, 0, 0), rad=1.0)
    assert R == ts.rotate(pos=0, axis=(1, 0, 0), angles=1.0)
    with pytest.warns(DeprecationWarning):
        R = ts.rotate(pos=0, axis=(1, 0, 0), deg=90.0)
    assert R == ts.rotate(pos=0, axis=(1, 0, 0), angles=np.pi / 2)
