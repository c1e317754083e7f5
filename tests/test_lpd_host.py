"""The learned primal-dual network's host structure on the CPU, with the
projector replaced by a small dense linear map and its transpose (the GPU
tests run it on the real projector): shapes, gradients reaching every block,
checkpointed gradients equal to stored ones, and the initial estimate."""
import pytest
import torch

from tomosipo_gb300 import lpd


class _Map:
    """y = M x over (batch, 1, *shape) tensors, a stand-in for A or A.T."""

    def __init__(self, M, domain, rng):
        self.M, self.domain_shape, self.range_shape = M, domain, rng

    @property
    def T(self):
        return _Map(self.M.T, self.range_shape, self.domain_shape)

    def __call__(self, x):
        flat = x.reshape(*x.shape[:2], -1) @ self.M.T
        return flat.reshape(*x.shape[:2], *self.range_shape)


@pytest.fixture
def net_factory(monkeypatch):
    monkeypatch.setattr(lpd, "to_autograd", lambda op, num_extra_dims: op)
    g = torch.Generator().manual_seed(0)
    A = _Map(torch.randn(4 * 3 * 5, 4 * 4 * 4, generator=g) / 8, (4, 4, 4), (4, 3, 5))

    def make(**kw):
        torch.manual_seed(1)
        return A, lpd.LearnedPrimalDual3d(A, channels=4, dtype=torch.float32, **kw)

    return make


def test_shapes_and_gradients_reach_every_block(net_factory):
    A, net = net_factory(n_iters=3)
    g = torch.randn(2, 1, *A.range_shape)
    out = net(g)
    assert out.shape == (2, 1, *A.domain_shape) and out.dtype == torch.float32
    out.square().mean().backward()
    for p in net.parameters():
        assert p.grad is not None and torch.isfinite(p.grad).all() and p.grad.abs().sum() > 0


def test_checkpointed_gradients_equal_stored_ones(net_factory):
    A, a = net_factory(n_iters=3, checkpoint=True)
    _, b = net_factory(n_iters=3, checkpoint=False)
    b.load_state_dict(a.state_dict())
    g = torch.randn(2, 1, *A.range_shape)
    for net in (a, b):
        net(g).square().sum().backward()
    for pa, pb in zip(a.parameters(), b.parameters()):
        assert torch.equal(pa.grad, pb.grad)


def test_initial_estimate_with_no_iterations_is_returned(net_factory):
    A, net = net_factory(n_iters=0)
    f0 = torch.randn(2, 1, *A.domain_shape)
    assert torch.equal(net(torch.randn(2, 1, *A.range_shape), f0), f0)


def test_unknown_activation_is_rejected(net_factory):
    with pytest.raises(ValueError):
        net_factory(n_iters=1, activation="tanh")
