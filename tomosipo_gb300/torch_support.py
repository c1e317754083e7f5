"""PyTorch autograd support (API of tomosipo's ``tomosipo/torch_support.py``).

``to_autograd(A, num_extra_dims=0, is_2d=False)`` wraps an operator (or its
transpose) in a hand-written ``torch.autograd.Function``: forward applies the
operator, backward applies its transpose. With the default matched
backprojector the transpose is the exact adjoint of the forward projector, so
gradients are exact to fp32 rounding (checked against central finite
differences in the tests). ``num_extra_dims`` leading batch/channel dimensions
are projected slice by slice into one preallocated fp32 output, as in the
reference (``torch_support.py:26-80``); ``is_2d`` drops the operator's first
(z) dimension. ``AutogradOperator`` / ``autograd_operator`` give an
operator-like object whose ``__call__`` and ``.T`` are differentiable.
"""
import itertools

import torch
from torch.autograd import Function

from .Operator import BackprojectionOperator, operator as make_operator


def _apply(op, x, out, extra_dims):
    """op over every slice of the leading ``extra_dims``. This package's
    operators take all slices of a CUDA tensor in one batched C-ABI call
    (tsgb_direct_fp_batch / tsgb_direct_bp_batch); other operators, and host
    data, go slice by slice as in the reference (torch_support.py:49-53)."""
    if len(extra_dims) == 0:
        op(x, out=out)
        return
    batch = getattr(op, "_apply_batch", None)
    if (batch is not None and x.is_cuda and out.is_cuda and x.dtype == torch.float32
            and x.is_contiguous() and out.is_contiguous()):
        n = 1
        for d in extra_dims:
            n *= d
        batch(x.reshape(n, *x.shape[len(extra_dims):]), out.reshape(n, *out.shape[len(extra_dims):]))
        return
    for idx in itertools.product(*[range(n) for n in extra_dims]):
        op(x[idx], out=out[idx])


class OperatorFunction(Function):
    """y = op(x) over ``num_extra_dims`` leading dimensions; dx = op.T(dy)."""

    @staticmethod
    def forward(ctx, input, operator, num_extra_dims=0, is_2d=False):
        extra_dims = tuple(input.shape[:num_extra_dims])
        expected_ndim = (2 if is_2d else 3) + num_extra_dims
        assert input.ndim == expected_ndim, (
            f"Tomosipo autograd operator expected {expected_ndim} dimensions "
            f"but got {input.ndim}.\n"
            "The interface of to_autograd was changed in Tomosipo 0.6.0 to "
            "by default match standard Tomosipo operators and extra arguments are "
            "provided to match Pytorch NN functions.\n"
            "To add batch and channel dimensions set argument num_extra_dims=2\n"
            "To remove the first operator dimension set argument is_2d=True\n"
        )
        ctx.operator = operator
        ctx.extra_dims = extra_dims
        ctx.is_2d = is_2d
        x = input.detach()
        if x.dtype != torch.float32:
            x = x.to(torch.float32)
        if is_2d:
            x = x.unsqueeze(-3)
        x = x.contiguous()
        out = torch.empty(extra_dims + tuple(operator.range_shape), dtype=torch.float32,
                          device=input.device)
        _apply(operator, x, out, extra_dims)
        if is_2d:
            out = out.squeeze(-3)
        return out

    @staticmethod
    def backward(ctx, grad_output):
        op = ctx.operator.T
        g = grad_output
        if g.dtype != torch.float32:
            g = g.to(torch.float32)
        if ctx.is_2d:
            g = g.unsqueeze(-3)
        g = g.contiguous()
        grad_input = torch.empty(ctx.extra_dims + tuple(op.range_shape), dtype=torch.float32,
                                 device=grad_output.device)
        _apply(op, g, grad_input, ctx.extra_dims)
        if ctx.is_2d:
            grad_input = grad_input.squeeze(-3)
        return grad_input, None, None, None


def to_autograd(operator, num_extra_dims=0, is_2d=False):
    """Differentiable function applying ``operator`` (``tomosipo/torch_support.py:83-130``)."""

    def f(x):
        return OperatorFunction.apply(x, operator, num_extra_dims, is_2d)

    return f


class AutogradOperator:
    """Operator-like object with differentiable ``__call__`` and ``.T``.

    Additive operators are rejected, as in the reference
    (``tomosipo/torch_support.py:239-240``).
    """

    def __init__(self, operator, num_extra_dims=0, is_2d=False):
        if operator.additive:
            raise ValueError("Additive operators are not supported")
        self.operator = operator
        self._fp_op = to_autograd(operator, num_extra_dims, is_2d)
        self._bp_op = to_autograd(operator.T, num_extra_dims, is_2d)
        self._transpose = BackprojectionOperator(self)

    def _fp(self, volume, out=None):
        if out is None:
            return self._fp_op(volume)
        out[...] = self._fp_op(volume)
        return out

    def _bp(self, projection, out=None):
        if out is None:
            return self._bp_op(projection)
        out[...] = self._bp_op(projection)
        return out

    def __call__(self, volume, out=None):
        return self._fp(volume, out)

    def transpose(self):
        return self._transpose

    @property
    def T(self):
        return self.transpose()

    @property
    def astra_compat_vg(self):
        return self.operator.astra_compat_vg

    @property
    def astra_compat_pg(self):
        return self.operator.astra_compat_pg

    @property
    def domain(self):
        return self.operator.domain

    @property
    def range(self):
        return self.operator.range

    @property
    def domain_shape(self):
        return self.operator.domain_shape

    @property
    def range_shape(self):
        return self.operator.range_shape


def autograd_operator(volume_geometry, projection_geometry, voxel_supersampling=1,
                      detector_supersampling=1, num_extra_dims=0, is_2d=False):
    """``AutogradOperator`` of a new operator (``tomosipo/torch_support.py:322-370``)."""
    op = make_operator(
        volume_geometry,
        projection_geometry,
        voxel_supersampling=voxel_supersampling,
        detector_supersampling=detector_supersampling,
    )
    return AutogradOperator(op, num_extra_dims=num_extra_dims, is_2d=is_2d)
