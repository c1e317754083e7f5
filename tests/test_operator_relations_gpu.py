"""The reference's relational operator tests, on this package's kernels.

tomosipo's own tests pin the projector through relations, not stored values
(``tests/test_Operator.py``): dataset and array inputs give the same result
(``:15-32``), an additive operator applied twice gives twice the projection
(``:35-49``), and moving the volume by a transform equals moving the
projection geometry by its inverse, for the forward projection and for the
backprojection of it (``:52-83``, over scalings x translations x rotations as
in ``tests/geometry/test_transform.py:16-52``; ``:86-112`` with a volume that
moves at every angle). The random transforms here are seeded.
"""
import itertools

import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300.Data import Data
from tests.helpers import TOL_ORACLE, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

_rng = np.random.default_rng(40)
SCALINGS = [ts.scale(1), ts.scale(abs(_rng.normal())), ts.scale(abs(_rng.normal(size=3)))]
TRANSLATIONS = [ts.translate((0, 0, 0)), ts.translate(_rng.normal(0, 1, size=3))]
ROTATIONS = [
    ts.rotate(pos=0, axis=(1, 0, 0), angles=0),
    ts.rotate(pos=0, axis=(1, 0, 0), angles=1.0),
    ts.rotate(pos=0, axis=_rng.normal(size=3), angles=_rng.normal()),
    ts.rotate(pos=0, axis=_rng.normal(size=3), angles=_rng.normal(), right_handed=False),
]


@pytest.fixture(scope="module")
def dev(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


def test_dataset_and_array_inputs(dev):
    pg = ts.cone(size=np.sqrt(2), cone_angle=1 / 2, angles=150, shape=100)
    vg = ts.volume(shape=100)
    A = ts.operator(vg, pg, additive=False)
    x = ts.phantom.hollow_box(ts.data(vg))
    y = A(x)
    assert isinstance(y, Data) and y.geometry == pg
    y_ = A(np.copy(x.data))  # array input
    assert np.sum(np.abs(y.data - y_)) == 0.0
    x1 = A.T(y)
    x2 = A.T(y.data)
    assert isinstance(x1, Data) and x1.geometry == vg
    assert np.sum(np.abs(x1.data - x2)) == 0.0


def test_additive_into_a_dataset(dev):
    pg = ts.cone(size=np.sqrt(2), cone_angle=1 / 2, angles=150, shape=100)
    vg = ts.volume(shape=100)
    A = ts.operator(vg, pg, additive=False)
    B = ts.operator(vg, pg, additive=True)
    x = ts.phantom.hollow_box(ts.data(vg))
    y = ts.data(pg)
    B(x, out=y)
    B(x, out=y)
    assert np.allclose(2 * A(x).data, y.data)


@pytest.mark.parametrize("S, T, R", list(itertools.product(SCALINGS, TRANSLATIONS, ROTATIONS)))
def test_moving_the_volume_equals_moving_the_detector(S, T, R, dev):
    pg = S * ts.parallel(angles=64, shape=96, size=1.5).to_vec()
    vg = S * ts.volume(shape=64, size=1)
    x = torch.from_numpy(
        np.random.default_rng(41).normal(size=(64, 64, 64)).astype(np.float32)).to(dev)
    A_v = ts.operator(T * R * vg.to_vec(), pg)
    A_p = ts.operator(vg, (T * R).inv * pg)
    yv, yp = A_v(x), A_p(x)
    assert rel_l2(yv.cpu().numpy(), yp.cpu().numpy()) <= TOL_ORACLE
    bv, bp = A_v.T(yv), A_p.T(yp)
    assert rel_l2(bv.cpu().numpy(), bp.cpu().numpy()) <= TOL_ORACLE


def test_volume_moving_at_every_angle(dev):
    pg = ts.parallel(angles=1, shape=48).to_vec()
    vg = ts.volume(shape=32)
    angles = np.linspace(0, np.pi, 48, endpoint=False)
    R = ts.rotate(pos=0, axis=(1, 0, 0), angles=angles)
    A_v = ts.operator(R * vg.to_vec(), pg)
    A_p = ts.operator(vg, R.inv * pg)
    x = torch.from_numpy(
        np.random.default_rng(42).normal(size=A_v.domain_shape).astype(np.float32)).to(dev)
    yv, yp = A_v(x), A_p(x)
    assert A_v.range_shape == (48, 48, 48)
    assert rel_l2(yv.cpu().numpy(), yp.cpu().numpy()) <= TOL_ORACLE
    assert rel_l2(A_v.T(yv).cpu().numpy(), A_p.T(yp).cpu().numpy()) <= TOL_ORACLE
