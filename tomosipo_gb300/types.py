"""Argument coercion for geometry constructors.

Accepts the same argument forms as tomosipo's ``tomosipo/types.py``
(scalars broadcast to tuples, ``(N, 3)`` vector arrays, homogeneous
coordinates), and raises ``TypeError`` on the same kinds of bad input.
Written for NumPy 2: no ``copy=False`` array construction.
"""
from collections import abc
from numbers import Integral

import numpy as np

EPSILON = 1e-8  # the package's ts.epsilon (tomosipo/__init__.py:41)


def _as_tuple(val, n):
    if isinstance(val, abc.Iterable) and not isinstance(val, (str, bytes)):
        val = tuple(val)
        if len(val) != n:
            raise TypeError(f"Expected tuple with {n} elements. Got {val!r}.")
        return val
    if isinstance(val, (str, bytes)):
        raise TypeError(f"Expected tuple with {n} elements. Got {val!r}.")
    return (val,) * n


def to_float_tuple(val, n, var_name="value"):
    val = _as_tuple(val, n)
    try:
        return tuple(float(v) for v in val)
    except (TypeError, ValueError):
        raise TypeError(f"{var_name} must contain only floats. Got {val!r}.")


def _to_shape(shape, n):
    shape = _as_tuple(shape, n)
    out = []
    for s in shape:
        if isinstance(s, (np.integer, Integral)) and not isinstance(s, bool):
            out.append(int(s))
        else:
            raise TypeError(
                f"Shape must contain only integers. Got {shape} with type {type(s)}.")
    if any(s < 1 for s in out):  # tomosipo/types.py:111-126: a TypeError, as for non-integers
        raise TypeError(f"Shape must be positive. Got {tuple(out)}.")
    return tuple(out)


def to_shape2d(shape):
    """(height, width) detector shape from an int or a pair."""
    return _to_shape(shape, 2)


def to_shape3d(shape):
    """(z, y, x) volume shape from an int or a triple."""
    return _to_shape(shape, 3)


def _to_size(size, n):
    size = to_float_tuple(size, n, "size")
    if any(s < -EPSILON for s in size):  # tomosipo/types.py:160-170
        raise TypeError(f"Size must be non-negative. Got {size}.")
    return size


# The reference's names for the n-dimensional forms (tomosipo/types.py:51-170).
to_tuple = _as_tuple
to_shape_nd = _to_shape
to_size_nd = _to_size


def to_size2d(size):
    return _to_size(size, 2)


def to_size3d(size):
    return _to_size(size, 3)


def to_pos(pos):
    """A 3-tuple of floats; the scalar 0 means the origin."""
    if np.isscalar(pos):
        if pos == 0.0:
            return (0.0, 0.0, 0.0)
        raise TypeError(f"Cannot convert {pos!r} to a position (z, y, x).")
    return to_float_tuple(pos, 3, "Position")


def to_scalars(s, var_name="scalars", accept_empty=False):
    """1-D float64 array from a float or a collection of floats."""
    try:
        arr = np.array(s, dtype=np.float64, ndmin=1)
    except (TypeError, ValueError):
        raise TypeError(f"Could not convert {var_name} to np.array. Got: {s!r}.")
    if np.any(np.isnan(arr)):
        raise TypeError("Could not convert to array of scalars: array contains NaN.")
    if arr.ndim == 1 and (accept_empty or len(arr) > 0):
        return arr
    raise TypeError(
        f"Value cannot be converted to {var_name}. "
        f"Expected shape: (N,). Got shape: {arr.shape}."
    )


def to_vec(vec, var_name="vector"):
    """(N, 3) float64 array from a 3-vector or a stack of 3-vectors."""
    try:
        arr = np.array(vec, dtype=np.float64)
    except (TypeError, ValueError):
        raise TypeError(f"Could not convert {var_name} to np.array. Got: {vec!r}.")
    shape = arr.shape
    arr = np.array(arr, ndmin=2)
    if arr.ndim == 2 and arr.shape[1] == 3:
        return arr
    raise TypeError(
        f"Value cannot be converted to {var_name}. "
        f"Expected shape: (3,) or (N, 3). Got shape: {shape}."
    )


def to_homogeneous(vec, s):
    """(N, 4) homogeneous coordinates; 3-vectors get ``s`` appended."""
    try:
        arr = np.array(vec, dtype=np.float64)
    except (TypeError, ValueError):
        raise TypeError(f"Could not convert value to np.array. Got: {vec!r}.")
    shape = arr.shape
    arr = np.array(arr, ndmin=2)
    if arr.ndim == 2 and arr.shape[1] == 4:
        return arr
    if arr.ndim == 2 and arr.shape[1] == 3:
        return np.concatenate([arr, np.full((arr.shape[0], 1), float(s))], axis=1)
    raise TypeError(
        "Value cannot be converted to homogeneous coordinates. "
        f"Expected shape: (3,), (4,), (N, 3), or (N, 4). Got shape: {shape}."
    )


def to_homogeneous_vec(vec):
    return to_homogeneous(vec, 0.0)


def to_homogeneous_pos(pos):
    return to_homogeneous(pos, 1.0)
