"""NumPy link (``tomosipo/links/numpy.py``): float32, C-contiguous host arrays.

Projections of NumPy data still run on the GPU: the data are staged to the
current CUDA device and the result copied back. There is no CPU compute path.
"""
import warnings

import numpy as np

from .base import Link, backends


class NumpyLink(Link):
    def __init__(self, shape, initial_value):
        super().__init__(shape, initial_value)
        if initial_value is None:
            self._data = np.zeros(shape, dtype=np.float32)
        elif np.isscalar(initial_value):
            self._data = np.full(shape, initial_value, dtype=np.float32)
        else:
            arr = np.asarray(initial_value)
            if arr.shape != tuple(shape):
                raise ValueError(
                    "Cannot link array. "
                    f"Expected array of shape {tuple(shape)}. Got {arr.shape}"
                )
            if arr.dtype != np.float32:
                warnings.warn(
                    f"The parameter initial_value is of type {arr.dtype}; expected `np.float32`. "
                    "The type has been Automatically converted. "
                    "Use `ts.link(x.astype(np.float32))' to inhibit this warning. "
                )
                arr = arr.astype(np.float32)
            if not (arr.flags["C_CONTIGUOUS"] and arr.flags["ALIGNED"]):
                warnings.warn(
                    "The parameter initial_value should be C_CONTIGUOUS and ALIGNED. "
                    "It has been automatically made contiguous and aligned. "
                    "Use `ts.link(np.ascontiguousarray(x))' to inhibit this warning. "
                )
                arr = np.ascontiguousarray(arr)
            self._data = arr

    @staticmethod
    def __accepts__(initial_value):
        return (
            initial_value is None
            or isinstance(initial_value, np.ndarray)
            or np.isscalar(initial_value)
        )

    def __compatible_with__(self, other):
        if isinstance(other, NumpyLink):
            return True
        return NotImplemented

    @property
    def linked_data(self):
        return self._data

    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, val):
        Link.data.fset(self, val)

    @property
    def is_cuda(self):
        return False

    def new_zeros(self, shape):
        return NumpyLink(shape, np.zeros(shape, dtype=self._data.dtype))

    def new_full(self, shape, value):
        return NumpyLink(shape, np.full(shape, value, dtype=self._data.dtype))

    def new_empty(self, shape):
        return NumpyLink(shape, np.empty(shape, dtype=self._data.dtype))

    def clone(self):
        return NumpyLink(self._data.shape, self._data.copy())


backends.append(NumpyLink)
