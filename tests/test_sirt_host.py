"""The plain SIRT recipe (``tomosipo_gb300.sirt.sirt``, ``README.md:150-163``
of the reference) on the CPU with a non-negative dense stand-in operator:
preconditioners clipped at 1 / epsilon, the first iteration's closed form,
and a monotonically falling residual on consistent data."""
import torch

from tomosipo_gb300.sirt import EPSILON, preconditioners, sirt


class _Dense:
    def __init__(self, M, domain, rng):
        self.M, self.domain_shape, self.range_shape = M, domain, rng

    @property
    def T(self):
        return _Dense(self.M.T, self.range_shape, self.domain_shape)

    def __call__(self, x, out=None):
        y = (self.M @ x.reshape(-1)).reshape(self.range_shape)
        if out is None:
            return y
        out[...] = y
        return out


def _operator():
    g = torch.Generator().manual_seed(0)
    M = torch.rand(2 * 6 * 3, 2 * 3 * 4, generator=g, dtype=torch.float64)
    M[M < 0.6] = 0  # sparse, like a projector
    M[5, :] = 0  # a ray that misses the volume
    M[:, 7] = 0  # a voxel no ray sees
    return _Dense(M.float(), (2, 3, 4), (2, 6, 3))


def test_preconditioners_are_clipped_reciprocals():
    A = _operator()
    R, C = preconditioners(A, "cpu")
    row, col = A.M.sum(1).reshape(A.range_shape), A.M.sum(0).reshape(A.domain_shape)
    assert torch.allclose(R, torch.clamp(1 / row, max=1 / EPSILON))
    assert torch.allclose(C, torch.clamp(1 / col, max=1 / EPSILON))
    assert R.reshape(-1)[5] == 1 / EPSILON and C.reshape(-1)[7] == 1 / EPSILON


def test_first_iteration_and_initial_estimate():
    A = _operator()
    R, C = preconditioners(A, "cpu")
    y = A(torch.rand(A.domain_shape))
    assert torch.allclose(sirt(A, y, 1), C * A.T(R * y))
    x0 = torch.rand(A.domain_shape)
    kept = x0.clone()
    x1 = sirt(A, y, 1, x_init=x0)
    assert torch.equal(x0, kept)  # the initial estimate is not modified
    assert torch.allclose(x1, x0 + C * A.T(R * (y - A(x0))))


def test_residual_falls_monotonically_on_consistent_data():
    A = _operator()
    x_true = torch.rand(A.domain_shape)
    x_true.reshape(-1)[7] = 0  # unseen by every ray
    y = A(x_true)
    R, _ = preconditioners(A, "cpu")
    R = torch.where(R == 1 / EPSILON, torch.zeros_like(R), R)  # weights of rays that exist
    x = torch.zeros(A.domain_shape)
    last = float("inf")
    for _ in range(30):
        x = sirt(A, y, 1, x_init=x)
        r = float(((y - A(x)) ** 2 * R).sum())  # SIRT descends this weighted norm
        assert r <= last * (1 + 1e-6)
        last = r
    assert last < 1e-2 * float((y ** 2 * R).sum())
