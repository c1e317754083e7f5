"""Interval slicing used by geometry ``__getitem__``.

Follows tomosipo's ``tomosipo/utils.py:45-119`` (``slice_interval``): a strided
slice keeps the centre of the first selected pixel and multiplies the pixel
size by the step, so slicing with a step bins pixels.
"""
from contextlib import contextmanager
from numbers import Integral

import numpy as np


def _to_slice(key, length):
    if isinstance(key, slice):
        return key
    if isinstance(key, (Integral, np.integer)):
        k = int(key)
        if k < 0:
            k += length
        if not 0 <= k < length:
            raise IndexError(f"Index {key} out of range for length {length}.")
        return slice(k, k + 1, 1)
    raise TypeError(f"Expected int or slice. Got {key!r}.")


def slice_interval(left, right, length, key):
    """Slice the interval [left, right] divided into ``length`` pixels.

    Returns ``(new_left, new_right, new_length, new_pixel_size)``.
    """
    pixel_size = 1 if length == 0 else (right - left) / length
    start, stop, step = _to_slice(key, length).indices(length)
    if step <= 0:
        raise ValueError("Only positive slice steps are supported on geometries.")
    new_len = max(0, -(-(stop - start) // step))
    new_pixel = pixel_size * step
    new_left = left + (start + 0.5) * pixel_size - 0.5 * new_pixel
    new_right = new_left + new_len * new_pixel
    return new_left, new_right, new_len, new_pixel


@contextmanager
def print_options():
    """Uniform NumPy print options (plain float reprs) for geometry ``__repr__``."""
    try:
        ctx = np.printoptions(legacy="1.25")
    except (TypeError, ValueError):  # older NumPy: default printing is already plain
        ctx = np.printoptions()
    with ctx:
        yield
