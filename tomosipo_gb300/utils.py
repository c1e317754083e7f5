"""Interval slicing used by geometry ``__getitem__``.

Follows tomosipo's ``tomosipo/utils.py:45-119`` (``slice_interval``): a strided
slice keeps the centre of the first selected pixel and multiplies the pixel
size by the step, so slicing with a step bins pixels.
"""
from contextlib import contextmanager
from numbers import Integral

import numpy as np


def up_slice(key):
    """An int index as the slice of one element (-1 as ``slice(-1, None)``)
    (``tomosipo/utils.py:35-42``); slices pass through."""
    if isinstance(key, (Integral, np.integer)):
        key = int(key)
        return slice(key, None) if key == -1 else slice(key, key + 1)
    if isinstance(key, slice):
        return key
    raise TypeError(f"Expected int or slice. Got {key!r}.")


def slice_interval(left, right, length, key):
    """Slice the interval [left, right] divided into ``length`` pixels.

    Returns ``(new_left, new_right, new_length, new_pixel_size)``: the
    selected pixels, each ``step`` times as wide as before and centred on
    the first pixel of its group, so a strided slice bins pixels. An
    interval of length 0 has pixel size 1.
    """
    pixel_size = 1 if length == 0 else (right - left) / length
    start, stop, step = up_slice(key).indices(length)
    if step <= 0:
        raise ValueError("Only positive slice steps are supported on geometries.")
    new_len = max(0, -(-(stop - start) // step))
    stop = max(start, start + (new_len - 1) * step + 1)  # one past the last pixel taken
    new_pixel = pixel_size * step
    new_left = left + start * pixel_size + 0.5 * pixel_size * (1 - step)
    new_right = left + stop * pixel_size + 0.5 * pixel_size * (step - 1)
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
