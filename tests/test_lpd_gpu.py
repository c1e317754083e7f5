"""Learned primal-dual on the projector: shapes, gradients by central finite
differences (eps = 1e-3, 16 random voxels), checkpointing (recompute instead of
store) equal to storing, and bf16 convolutions training."""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300.lpd import LearnedPrimalDual3d

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.fixture
def exact_convs():
    """fp32 convolutions without TF32 and with deterministic algorithms, so
    finite differences and recomputation compare like with like."""
    b = torch.backends.cudnn
    old = (b.allow_tf32, b.deterministic, b.benchmark, torch.backends.cuda.matmul.allow_tf32)
    b.allow_tf32, b.deterministic, b.benchmark = False, True, False
    torch.backends.cuda.matmul.allow_tf32 = False
    yield
    b.allow_tf32, b.deterministic, b.benchmark, torch.backends.cuda.matmul.allow_tf32 = old


def _setup(dev, n=24, angles=24, dtype=torch.float32, iters=2, channels=8, checkpoint=True,
           activation="relu"):
    vg = ts.volume(shape=n, size=1)
    pg = ts.cone(angles=angles, shape=(n, 3 * n // 2), size=np.sqrt(2), cone_angle=0.5)
    A = ts.operator(vg, pg)
    torch.manual_seed(0)
    net = LearnedPrimalDual3d(A, n_iters=iters, channels=channels, dtype=dtype,
                              checkpoint=checkpoint, activation=activation).to(dev)
    return A, net


def test_forward_backward_bf16(dev):
    A, net = _setup(dev, dtype=torch.bfloat16)
    g = torch.rand(2, 1, *A.range_shape, device=dev)
    out = net(g)
    assert out.shape == (2, 1, *A.domain_shape) and out.dtype == torch.float32
    out.square().mean().backward()
    assert all(p.grad is not None and torch.isfinite(p.grad.float()).all() for p in net.parameters())


def test_checkpoint_equals_stored_activations(dev, exact_convs):
    A, net = _setup(dev, checkpoint=True)
    g = torch.rand(2, 1, *A.range_shape, device=dev)
    net(g).square().sum().backward()
    grads_ckpt = [p.grad.clone() for p in net.parameters()]
    net.zero_grad()
    net.use_checkpoint = False
    net(g).square().sum().backward()
    for a, b in zip(grads_ckpt, (p.grad for p in net.parameters())):
        assert torch.equal(a, b)


@pytest.mark.parametrize("activation,rel,abs_", [("relu", 5e-2, 5e-3), ("softplus", 2e-2, 1e-3)])
def test_gradient_central_differences_16_voxels(dev, exact_convs, activation, rel, abs_):
    """d/d f0_i of sum(w * LPD(g, f0)) by central differences (eps = 1e-3) on 16
    random voxels, fp32 network. The band is rel |grad| + abs plus half the gap
    between the two one-sided differences: in an fp32 network that gap is the
    rounding noise of the differences themselves (about 1e-2 at eps = 1e-3, so
    a few 1e-3 on the central difference), and it stays small for a smooth
    network. With ReLU a perturbation can cross a kink, where the central
    difference is no derivative at all: a voxel whose one-sided differences
    disagree beyond twice the band is such a crossing and is left out (at most
    3 of 16); the band is also wider. The smooth network is checked on all 16."""
    A, net = _setup(dev, dtype=torch.float32, activation=activation)
    gen = torch.Generator(device="cpu").manual_seed(1)
    g = torch.rand(1, 1, *A.range_shape, generator=gen).to(dev)
    f0 = torch.rand(1, 1, *A.domain_shape, generator=gen).to(dev).requires_grad_(True)
    w = torch.rand(1, 1, *A.domain_shape, generator=gen).to(dev)
    (net(g, f0) * w).sum().backward()
    eps = 1e-3
    idx = torch.randint(0, f0.numel(), (16,), generator=gen).tolist()
    bad = kinks = 0
    report = []
    with torch.no_grad():
        l0 = (net(g, f0).double() * w.double()).sum()
        for i in idx:
            e = torch.zeros(f0.numel(), device=dev)
            e[i] = eps
            e = e.view_as(f0)
            lp = (net(g, f0 + e).double() * w.double()).sum()
            lm = (net(g, f0 - e).double() * w.double()).sum()
            fd = float((lp - lm) / (2 * eps))
            an = float(f0.grad.view(-1)[i])
            band = rel * abs(an) + abs_
            gap = abs(float((lp - l0) - (l0 - lm)) / eps)
            report.append((round(an, 5), round(fd, 5), round(gap, 5)))
            if activation == "relu" and gap > 2 * band:
                kinks += 1  # one-sided slopes differ: a kink lies within +-eps
                continue
            if abs(fd - an) > band + 0.5 * gap:
                bad += 1
    assert bad == 0 and kinks <= 3, (bad, kinks, report)
