"""ts.data and the legacy projection functions' host side (tomosipo's
tests/test_Data.py and tests/test_astra.py behaviour that needs no GPU)."""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300.astra import backward, fdk, forward, project


def test_init_warns_and_rejects_like_the_reference():
    pg = ts.cone(angles=10, shape=20, cone_angle=1 / 2)
    vg = ts.volume().reshape(10)
    pd = ts.data(pg, 0)
    shape = pd.data.shape
    assert shape == (20, 10, 20)
    with pytest.warns(UserWarning):
        ts.data(pg, np.ones(shape, dtype=np.float64))
    with pytest.warns(UserWarning):
        ts.data(vg, np.ones(vg.shape, dtype=np.float64))
    with pytest.warns(UserWarning):
        p = np.ones((shape[0] * 2, shape[1], shape[2]), dtype=np.float32)
        ts.data(pg, p[::2, ...])
    with pytest.raises(TypeError):
        ts.data(vg.to_vec())
    ts.data(pg, np.ones(shape, dtype=np.float32))


def test_with_data_and_predicates():
    pg = ts.cone(size=np.sqrt(2), cone_angle=1 / 2).reshape(10)
    vg = ts.volume()
    with ts.data(pg, 0) as pd, ts.data(vg, 0) as vd:
        assert np.all(abs(pd.data) < ts.epsilon)
        pd.data[:] = 1.0
        assert np.all(abs(pd.data - 1) < ts.epsilon)
        assert pd.is_projection() and not pd.is_volume()
        assert vd.is_volume() and not vd.is_projection()


def test_idempotent_and_clone():
    vg = ts.volume(shape=4)
    d = ts.data(vg, 2.0)
    assert ts.data(vg, d) is d
    with pytest.raises(ValueError):
        ts.data(ts.volume(shape=5), d)
    c = d.clone()
    c.data[:] = 3.0
    assert np.all(d.data == 2.0) and np.all(c.data == 3.0)


def test_project_argument_errors():
    vd = ts.data(ts.volume(shape=4))
    pd = ts.data(ts.cone(angles=2, shape=4, cone_angle=0.5))
    with pytest.raises(ValueError):
        project(vd, pd)
    with pytest.raises(ValueError):
        forward(vd)
    with pytest.raises(ValueError):
        backward(pd)
    with pytest.raises(ValueError):
        fdk(ts.data(ts.volume(shape=4)), ts.data(ts.parallel(angles=2, shape=4)))


def test_volume_contiguity_warning_and_projection_idempotency():
    """tests/test_Data.py:31-34, 75-107: a strided volume is copied with a warning;
    ``ts.data`` returns the dataset itself for an equal (not identical) geometry and
    rejects a dataset of another geometry."""
    vg = ts.volume().reshape(10)
    with pytest.warns(UserWarning):
        ts.data(vg, np.ones((20, 10, 10), dtype=np.float32)[::2, ...])
    pd = ts.data(ts.cone(size=np.sqrt(2), cone_angle=1 / 2, angles=10, shape=20))
    equal = ts.cone(size=np.sqrt(2), cone_angle=1 / 2, angles=10, shape=20)
    assert ts.data(equal, pd) is pd
    for other in (ts.volume(shape=10), ts.cone(size=np.sqrt(2), cone_angle=1 / 2)):
        with pytest.raises(ValueError):
            ts.data(other, pd)
