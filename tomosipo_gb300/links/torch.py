"""PyTorch link (``tomosipo/links/torch.py``).

A scalar fills a new float32 tensor; other tensors must have the expected
shape and are converted to float32 and made contiguous with a warning
(``tomosipo/links/torch.py:43-68``). CUDA tensors are projected in place on
their own device and on that device's current stream.
"""
import warnings
from contextlib import contextmanager

import torch

from .base import Link, backends
from .numpy import NumpyLink


class TorchLink(Link):
    def __init__(self, shape, initial_value):
        super().__init__(shape, initial_value)
        if not isinstance(initial_value, torch.Tensor):
            raise ValueError(
                f"Expected initial_value to be a `torch.Tensor'. Got {initial_value.__class__}"
            )
        if initial_value.shape == torch.Size([]):
            data = torch.zeros(shape, dtype=torch.float32, device=initial_value.device)
            data[...] = initial_value
            self._data = data
            return
        if tuple(initial_value.shape) != tuple(shape):
            raise ValueError(
                f"Expected initial_value with shape {tuple(shape)}. Got {tuple(initial_value.shape)}"
            )
        if initial_value.dtype != torch.float32:
            warnings.warn(
                f"The parameter initial_value is of type {initial_value.dtype}; expected "
                "`torch.float32`. The type has been automatically converted. "
                "Use `ts.link(x.to(dtype=torch.float32))' to inhibit this warning. "
            )
            initial_value = initial_value.to(dtype=torch.float32)
        if not initial_value.is_contiguous():
            warnings.warn(
                "The parameter initial_value should be contiguous. "
                "It has been automatically made contiguous. "
                "Use `ts.link(x.contiguous())' to inhibit this warning. "
            )
            initial_value = initial_value.contiguous()
        self._data = initial_value

    @staticmethod
    def __accepts__(initial_value):
        return isinstance(initial_value, torch.Tensor)

    def __compatible_with__(self, other):
        if isinstance(other, NumpyLink):
            other_dev = torch.device("cpu")
        elif isinstance(other, TorchLink):
            other_dev = other._data.device
        else:
            return NotImplemented
        return self._data.device == other_dev

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
        return self._data.is_cuda

    @contextmanager
    def context(self):
        if self._data.is_cuda:
            with torch.cuda.device_of(self._data):
                yield
        else:
            yield

    def new_zeros(self, shape):
        return TorchLink(shape, self._data.new_zeros(shape))

    def new_full(self, shape, value):
        return TorchLink(shape, self._data.new_full(shape, value))

    def new_empty(self, shape):
        return TorchLink(shape, self._data.new_empty(shape))

    def clone(self):
        return TorchLink(self._data.shape, self._data.clone())


backends.insert(0, TorchLink)
