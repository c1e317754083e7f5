"""Interval slicing and vector broadcasting behind geometry indexing, and the
argument coercions of the geometry constructors (tomosipo's
``tests/test_utils.py``, ``tests/test_vector_calc.py``,
``tests/links/test_numpy.py``, and the examples that ``tests/test_types.py``
runs from ``tomosipo/types.py``), restated. Host only.
"""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300 import vector_calc as vc
from tomosipo_gb300.utils import slice_interval


class Interval:
    """A 1-D pixel interval [l, r] of `length` pixels, sliced like an axis."""

    def __init__(self, l, r, length):
        self.l, self.r, self.length = l, r, length

    def __getitem__(self, key):
        l, r, length, _ = slice_interval(self.l, self.r, self.length, key)
        return Interval(l, r, length)

    def __eq__(self, other):
        return (self.length == other.length and np.all(abs(self.l - other.l) < ts.epsilon)
                and np.all(abs(self.r - other.r) < ts.epsilon))

    size = property(lambda self: self.r - self.l)
    pixel_size = property(lambda self: self.size / self.length)
    center_of_left_pixel = property(lambda self: self.l + self.pixel_size / 2)
    center = property(lambda self: (self.l + self.r) / 2)


def test_slice_interval_basic_cases():
    assert slice_interval(0, 1, 1, 0) == (0, 1, 1, 1)
    assert slice_interval(0, 1, 1, slice(None)) == (0, 1, 1, 1)
    assert slice_interval(0, 0, 1, 0) == (0, 0, 1, 0)
    assert slice_interval(0, 0, 0, 0) == (0, 0, 0, 1)
    l0, r0 = np.arange(10), np.arange(10) + 1
    l1, r1, length1, _ = slice_interval(l0, r0, 10, slice(None))
    assert np.abs(l0 - l1).sum() == pytest.approx(0) and np.abs(r0 - r1).sum() == pytest.approx(0)
    assert length1 == 10


def test_slice_interval_steps_and_offsets():
    st = Interval(0, 10, 10)
    for i in range(1, 5):  # a start offset translates the sliced interval
        assert st[::5] != st[i::5] and st[::5].length == st[i::5].length
        assert st[::5].l + i == pytest.approx(st[i::5].l)
        assert st[::5].r + i == pytest.approx(st[i::5].r)
        assert st[::5].center + i == pytest.approx(st[i::5].center)
        assert st[::5].size == st[i::5].size
    for step in range(1, 10):  # the left-most pixel's centre stays put
        assert st[::step].center_of_left_pixel == pytest.approx(st.center_of_left_pixel)
    for length in (0, 5, 6):  # lengths as NumPy slicing counts them
        st = Interval(0, 1, length)
        ones = np.ones(length)
        for start in range(length):
            for step in (1, 2, 3, 4):
                assert st[start::step].length == len(ones[start::step])
                assert st[start::step].pixel_size == pytest.approx(step * st.pixel_size)
    st = Interval(0, 1, 30)
    assert st[::2].pixel_size == pytest.approx(2 * st.pixel_size)
    assert st[1::2].size == pytest.approx(1.0) and st[2::3].size == pytest.approx(1.0)
    assert st[4::5].size == pytest.approx(1.0)
    assert st[1::3].center == pytest.approx(st.center)
    assert st[0::3].center != pytest.approx(st.center)
    assert st[2::3].center != pytest.approx(st.center)


def test_vector_broadcasting():
    assert vc.broadcast_lengths(1, 1) == 1 and vc.broadcast_lengths(1, 5) == 5
    assert vc.broadcast_lengths(5, 1) == 5 and vc.broadcast_lengths(3, 3) == 3
    with pytest.raises(ValueError):
        vc.broadcast_lengths(2, 3)
    for a, b in (((3,), (3,)), ((1, 3), (3,)), ((1, 3), (1, 3)), ((3,), (1, 3))):
        x, y = vc._broadcastv(np.ones(a), np.ones(b))
        assert x.shape == y.shape == (1, 3)
    for a, b in (((1, 1, 3), (1, 3)), ((1, 3), (1, 1, 3)), ((2, 3), (3, 3))):
        with pytest.raises(ValueError):
            vc._broadcastv(np.ones(a), np.ones(b))
    A, B = vc._broadcastmm(np.ones((1, 2, 11)), np.ones((1, 11, 3)))
    assert A.shape == (1, 2, 11) and B.shape == (1, 11, 3)
    assert vc.matrix_matrix_transform(A, B).shape == (1, 2, 3)
    with pytest.raises(ValueError):
        vc._broadcastmm(np.ones((2, 3, 3)), np.ones((3, 3, 3)))
    assert vc.matrix_transform(np.ones((2, 3, 11)), np.ones((1, 11))).shape == (2, 3)


def test_numpy_link_checks_the_shape():
    with pytest.raises(ValueError):
        ts.link(ts.volume(shape=10), np.zeros((9, 9, 9), dtype=np.float32))


def test_type_coercion_names_and_errors():
    from tomosipo_gb300 import types

    assert types.to_tuple(1, 2) == (1, 1) and types.to_tuple((1, 2), n=2) == (1, 2)
    with pytest.raises(TypeError, match="Expected tuple with 2 elements"):
        types.to_tuple((1, 2, 3), n=2)
    assert types.to_shape2d(1) == (1, 1) and types.to_shape2d((5, 3)) == (5, 3)
    with pytest.raises(TypeError, match="with type <class 'float'>"):
        types.to_shape2d((5.0, 3))
    with pytest.raises(TypeError):
        types.to_shape3d((5, 3))
    assert types.to_shape_nd(2, 4) == (2, 2, 2, 2)
    assert types.to_size_nd(1.5, 2) == (1.5, 1.5)
    with pytest.raises(TypeError):
        types.to_size2d(-1)


def test_link_coercion_rules():
    """Links coerce to contiguous fp32 with a UserWarning, reject wrong shapes
    and unsupported types (tomosipo/links/numpy.py, links/torch.py)."""
    import warnings

    torch = pytest.importorskip("torch")
    vg = ts.volume(shape=4)
    quiet = [np.zeros((4, 4, 4), np.float32), torch.zeros(4, 4, 4)]
    noisy = [np.zeros((4, 4, 4)), np.zeros((8, 4, 4), np.float32)[::2],
             torch.zeros(4, 4, 4, dtype=torch.float64), torch.zeros(8, 4, 4)[::2]]
    for x in quiet:
        with warnings.catch_warnings():
            warnings.simplefilter("error")
            link = ts.link(vg, x)
        assert link.data.dtype in (np.float32, torch.float32)
    for x in noisy:
        with pytest.warns(UserWarning):
            link = ts.link(vg, x)
        assert link.data.dtype in (np.float32, torch.float32)
        assert (link.data.flags["C_CONTIGUOUS"] if isinstance(link.data, np.ndarray)
                else link.data.is_contiguous())
    with pytest.raises(ValueError):
        ts.link(vg, torch.zeros(3, 4, 4))
    with pytest.raises(ValueError):
        ts.link(vg, [1, 2, 3])


_COERCION_ERRORS = [  # the messages tomosipo/types.py documents for each coercion
    ("to_float_tuple", (("a", 0), 2), "value must contain only floats. Got ('a', 0)."),
    ("to_size2d", ((3, 2, 1),), "Expected tuple with 2 elements. Got (3, 2, 1)."),
    ("to_size3d", ((2, 1),), "Expected tuple with 3 elements. Got (2, 1)."),
    ("to_pos", ((2, 1),), "Expected tuple with 3 elements. Got (2, 1)."),
    ("to_scalars", (np.ones((1, 3)),),
     "Value cannot be converted to scalars. Expected shape: (N,). Got shape: (1, 3)."),
    ("to_scalars", ([],),
     "Value cannot be converted to scalars. Expected shape: (N,). Got shape: (0,)."),
    ("to_scalars", ("string",), "Could not convert scalars to np.array. Got: 'string'."),
    ("to_scalars", (None,), "Could not convert to array of scalars: array contains NaN."),
    ("to_vec", (np.ones((1, 2)),),
     "Value cannot be converted to vector. Expected shape: (3,) or (N, 3). Got shape: (1, 2)."),
    ("to_vec", ("string",), "Could not convert vector to np.array. Got: 'string'."),
]


@pytest.mark.parametrize("name, args, message", _COERCION_ERRORS)
def test_coercion_error_messages(name, args, message):
    import re

    from tomosipo_gb300 import types

    with pytest.raises(TypeError, match=re.escape(message)):
        getattr(types, name)(*args)


def test_coercion_values():
    from tomosipo_gb300 import types

    assert types.to_float_tuple(1, n=2) == (1.0, 1.0)
    assert types.to_float_tuple((1.0, 2.0), n=2) == (1.0, 2.0)
    assert types.to_shape3d(1) == (1, 1, 1) and types.to_shape3d((5, 3, 2)) == (5, 3, 2)
    assert types.to_size2d((5, 3)) == (5.0, 3.0) and types.to_size3d(1) == (1.0, 1.0, 1.0)
    assert types.to_pos(0) == types.to_pos(0.0) == (0.0, 0.0, 0.0)
    assert types.to_pos((3, 2, 1)) == (3.0, 2.0, 1.0)
    assert types.to_scalars(1).shape == (1,)
    assert np.array_equal(types.to_scalars((1, 1, 1)), np.ones(3))
    assert types.to_scalars([], accept_empty=True).shape == (0,)
    assert types.to_vec((1, 1, 1)).shape == (1, 3)
    assert types.to_vec([(1, 1, 1), (2, 2, 2)]).shape == (2, 3)
    assert types.to_vec(np.ones((1, 3))).shape == (1, 3)


def test_link_allocates_like_its_data():
    """tests/test_torch_support.py:32-43: a link's new_zeros / new_full / new_empty
    give links of the same kind, values and shape (host arrays here)."""
    torch = pytest.importorskip("torch")
    vg = ts.volume(shape=8)
    A = ts.operator(vg, ts.parallel(angles=12, shape=(8, 12)))
    for vol in (torch.zeros(A.domain_shape), np.zeros(A.domain_shape, dtype=np.float32)):
        link = ts.link(vg, vol)
        zeros, full = link.new_zeros(A.domain_shape), link.new_full(A.domain_shape, 1.0)
        assert type(zeros) is type(link) and type(zeros.data) is type(vol)
        assert np.allclose(np.asarray(zeros.data), np.asarray(vol))
        assert np.allclose(np.asarray(full.data), np.asarray(vol) + 1.0)
        assert link.new_empty(A.domain_shape).shape == link.shape
