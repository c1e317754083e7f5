"""``to_autograd`` / ``AutogradOperator`` host logic on the CPU, with a dense
stand-in operator (tomosipo's ``tests/test_torch_support.py`` rules; the GPU
tests run the same rules on the real projector): fp32 output for any input
dtype, slice-by-slice extra dimensions, ``is_2d``, gradients = the transpose,
dimension errors and the additive-operator rule."""
import pytest
import torch

from tomosipo_gb300.torch_support import AutogradOperator, to_autograd


class _Dense:
    """A linear operator y = M x on fixed shapes, with ``out=`` and ``.T``."""

    def __init__(self, M, domain, rng, additive=False):
        self.M, self.domain_shape, self.range_shape, self.additive = M, domain, rng, additive
        self.calls = 0

    @property
    def T(self):
        return _Dense(self.M.T, self.range_shape, self.domain_shape)

    def __call__(self, x, out=None):
        assert x.dtype == torch.float32 and x.is_contiguous() and tuple(x.shape) == self.domain_shape
        self.calls += 1
        y = (self.M @ x.reshape(-1)).reshape(self.range_shape)
        if out is None:
            return y
        out[...] = y
        return out


def _operator(domain=(2, 3, 4), rng=(2, 5, 3)):
    n, m = torch.Size(domain).numel(), torch.Size(rng).numel()
    return _Dense(torch.randn(m, n, generator=torch.Generator().manual_seed(0)), domain, rng)


def test_any_input_dtype_gives_fp32():
    A = _operator()
    x = torch.rand(A.domain_shape, dtype=torch.float64)
    y = to_autograd(A)(x)
    assert y.dtype == torch.float32 and torch.equal(y, A(x.float()))


def test_extra_dimensions_are_projected_slice_by_slice():
    A = _operator()
    x = torch.rand(2, 3, *A.domain_shape)
    y = to_autograd(A, num_extra_dims=2)(x)
    assert y.shape == (2, 3, *A.range_shape) and A.calls == 2 * 3
    for i in range(2):
        for j in range(3):
            assert torch.equal(y[i, j], A(x[i, j]))


def test_gradient_is_the_transpose():
    A = _operator()
    x = torch.rand(4, *A.domain_shape, requires_grad=True)
    y = to_autograd(A, num_extra_dims=1)(x)
    y.backward(y)
    expected = torch.stack([A.T(A(x[k].detach())) for k in range(4)])
    assert torch.allclose(x.grad, expected, rtol=1e-5, atol=1e-5)


def test_is_2d_drops_the_first_operator_dimension():
    A = _operator(domain=(1, 3, 4), rng=(1, 5, 3))
    x = torch.rand(2, 1, 3, 4, requires_grad=True)
    y = to_autograd(A, num_extra_dims=2, is_2d=True)(x)
    assert y.shape == (2, 1, 5, 3)
    y.sum().backward()
    assert x.grad.shape == x.shape


def test_wrong_number_of_dimensions_is_explained():
    A = _operator()
    with pytest.raises(AssertionError, match="num_extra_dims=2"):
        to_autograd(A)(torch.rand(1, *A.domain_shape))


def test_autograd_operator_rules():
    A = _operator()
    with pytest.raises(ValueError, match="Additive"):
        AutogradOperator(_Dense(A.M, A.domain_shape, A.range_shape, additive=True))
    op = AutogradOperator(A)
    assert op.domain_shape == A.domain_shape and op.range_shape == A.range_shape
    x = torch.rand(A.domain_shape, requires_grad=True)
    y = op(x)
    out = torch.empty(A.domain_shape)
    assert op.T(y.detach(), out=out) is out and torch.allclose(out, A.T(y.detach()))
    op.T(y).sum().backward()  # differentiable through both directions
    assert x.grad.shape == x.shape
