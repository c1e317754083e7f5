"""Device-array link: the role of tomosipo's CuPy link (``tomosipo/links/cupy.py``).

Any object that exposes ``__cuda_array_interface__`` and is not a torch tensor
(a CuPy array, a Numba device array, ...) is projected in place through a
zero-copy torch view of its memory. New outputs (``A(x)`` without ``out=``)
are CuPy arrays when CuPy is importable, else torch tensors on the same
device. As in the reference, arrays that are not float32 or not C-contiguous
are converted, with a warning, and the converted copy is what gets projected.
The reference registers its CuPy link on ``import tomosipo.cupy``; this one is
registered when ``tomosipo_gb300`` is imported (``tomosipo_gb300.cupy``
exists for scripts that import it).
"""
import warnings

import torch

from .base import Link, backends
from .numpy import NumpyLink
from .torch import TorchLink


def _device_array(t):
    """A CuPy array sharing ``t``'s memory if CuPy is importable, else ``t``."""
    try:
        import cupy
    except ImportError:
        return t
    return cupy.asarray(t)  # keeps a reference to t (the memory's owner)


class CudaArrayLink(Link):
    def __init__(self, shape, initial_value):
        super().__init__(shape, initial_value)
        if not CudaArrayLink.__accepts__(initial_value):
            raise ValueError(
                "Expected an object with __cuda_array_interface__. "
                f"Got {initial_value.__class__}"
            )
        view = torch.as_tensor(initial_value)  # zero copy, on the array's own device
        if not view.is_cuda:
            raise ValueError("the array interface does not describe device memory")
        if tuple(view.shape) != tuple(shape):
            raise ValueError(f"Expected initial_value with shape {tuple(shape)}. Got {tuple(view.shape)}")
        data = initial_value
        if view.dtype != torch.float32:
            warnings.warn(
                f"The parameter initial_value is of type {view.dtype}; expected float32. "
                "The type has been automatically converted. "
                "Use `ts.link(x.astype('float32'))' to inhibit this warning. "
            )
            view = view.to(torch.float32)
            data = _device_array(view)
        if not view.is_contiguous():
            warnings.warn(
                "The parameter initial_value should be C_CONTIGUOUS. "
                "It has been automatically made contiguous. "
                "Use `ts.link(cupy.ascontiguousarray(x))' to inhibit this warning. "
            )
            view = view.contiguous()
            data = _device_array(view)
        self._data = data
        self._view = view

    @staticmethod
    def __accepts__(initial_value):
        return hasattr(initial_value, "__cuda_array_interface__") and not isinstance(
            initial_value, torch.Tensor)

    def __compatible_with__(self, other):
        dev = self._view.device
        if isinstance(other, CudaArrayLink):
            return dev == other._view.device
        if isinstance(other, TorchLink):
            return dev == other.data.device
        if isinstance(other, NumpyLink):
            return False
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
    def torch_view(self):
        """float32 contiguous CUDA tensor sharing the projected memory."""
        return self._view

    @property
    def is_cuda(self):
        return True

    def _new(self, shape, t):
        arr = _device_array(t)
        return CudaArrayLink(shape, arr) if arr is not t else TorchLink(shape, t)

    def new_zeros(self, shape):
        return self._new(shape, self._view.new_zeros(shape))

    def new_full(self, shape, value):
        return self._new(shape, self._view.new_full(shape, value))

    def new_empty(self, shape):
        return self._new(shape, self._view.new_empty(shape))

    def clone(self):
        return self._new(self._view.shape, self._view.clone())


backends.append(CudaArrayLink)
