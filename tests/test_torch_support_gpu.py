"""Autograd support, ported from the reference's tests/test_torch_support.py plus
gradient checks by central finite differences (the matched backprojector is the
exact adjoint, so the gradient of <w, A x> is A^T w)."""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300.torch_support import AutogradOperator, autograd_operator, to_autograd

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = 64
N_angles = N * 3 // 2
M = N * 3 // 2


@pytest.fixture(scope="module")
def dev(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)


@pytest.mark.parametrize("device", ["cpu", "cuda"])
def test_fp_bp_positive(dev, device):
    # tests/test_torch_support.py:62-74
    vg = ts.volume(shape=N)
    pg = ts.parallel(angles=N_angles, shape=(N, M))
    A = ts.operator(vg, pg)
    vol = torch.ones(A.domain_shape).to(device)
    sino = A(vol)
    bp = A.T(sino)
    assert sino.device == vol.device and bp.device == vol.device
    assert 1.0 < sino.sum() and 1.0 < bp.sum()


def test_float64(dev):
    # :77-88 -- a float64 input gives the same fp32 output as the plain operator
    vg = ts.volume(shape=(1, N, N))
    pg = ts.parallel(angles=N_angles, shape=(1, M))
    A = ts.operator(vg, pg)
    A_ag = to_autograd(A)
    x = torch.ones((1, N, N), dtype=torch.float64, device=dev)
    with pytest.warns(UserWarning):
        y = A(x)
    y_ag = A_ag(x)
    assert y_ag.dtype == torch.float32
    assert torch.equal(y, y_ag)


def test_autograd(dev):
    # :91-100 -- x.grad == A.T(A(x)) for y.backward(y)
    vg = ts.volume(shape=(1, N, N))
    pg = ts.parallel(angles=N_angles, shape=(1, M))
    A = ts.operator(vg, pg)
    A_ag = to_autograd(A)
    x = torch.ones(A.domain_shape, dtype=torch.float32, device=dev, requires_grad=True)
    y = A_ag(x)
    y.backward(y)
    assert torch.allclose(x.grad, A.T(A(x.detach())))


def test_autograd_shape(dev):
    # :103-120
    vg = ts.volume(shape=(1, N, N))
    pg = ts.parallel(angles=N_angles, shape=(1, M))
    A = ts.operator(vg, pg)
    A_ag = to_autograd(A, num_extra_dims=2)
    x1 = torch.ones(1, 1, *A.domain_shape, device=dev, requires_grad=True)
    x2 = torch.ones(2, 3, *A.domain_shape, device=dev, requires_grad=True)
    y1, y2 = A_ag(x1), A_ag(x2)
    y1.backward(y1)
    y2.backward(y2)
    assert tuple(y1.shape) == (1, 1, *A.range_shape)
    assert tuple(y2.shape) == (2, 3, *A.range_shape)
    assert tuple(x1.grad.shape) == (1, 1, *A.domain_shape)
    assert tuple(x2.grad.shape) == (2, 3, *A.domain_shape)
    # every slice is the plain operator applied to that slice
    assert torch.equal(y2[1, 2], A(x2.detach()[1, 2]))


def test_is_2d(dev):
    vg = ts.volume(shape=(1, N, N))
    pg = ts.parallel(angles=N_angles, shape=(1, M))
    A = ts.operator(vg, pg)
    f = to_autograd(A, num_extra_dims=2, is_2d=True)
    x = torch.rand(4, 1, N, N, device=dev, requires_grad=True)
    y = f(x)
    assert tuple(y.shape) == (4, 1, N_angles, M)
    y.sum().backward()
    assert tuple(x.grad.shape) == (4, 1, N, N)
    assert torch.equal(y[2, 0], A(x.detach()[2, 0][None])[0])


def test_autograd_operator(dev):
    # :123-157
    vg = ts.volume(shape=(1, N, N))
    pg = ts.parallel(angles=N_angles, shape=(1, M))
    A = ts.operator(vg, pg)
    x = torch.zeros(A.domain_shape, dtype=torch.float32, device=dev)
    x[:, 10:-10, 10:-10] = 1.0
    x[:, 20:-20, 20:-20] = 0.0
    for A_ag in [AutogradOperator(A), autograd_operator(vg, pg)]:
        y, b = A(x), A.T(A(x))
        y2 = A(b)
        y_ag = A_ag(x)
        b_ag = A_ag.T(y_ag)
        y2_ag = A_ag(b_ag)
        assert torch.equal(y, y_ag) and torch.equal(b, b_ag) and torch.equal(y2, y2_ag)
        y_ag[...] = 0
        b_ag[...] = 0
        y2_ag[...] = 0
        A_ag(x, out=y_ag)
        A_ag.T(y_ag, out=b_ag)
        A_ag(b_ag, out=y2_ag)
        assert torch.equal(y, y_ag) and torch.equal(b, b_ag) and torch.equal(y2, y2_ag)
    with pytest.raises(ValueError):
        AutogradOperator(ts.operator(vg, pg, additive=True))


def test_autograd_operator_backward(dev):
    # :160-174
    vg = ts.volume(shape=(1, N, N))
    pg = ts.parallel(angles=N_angles, shape=(1, M))
    A = ts.operator(vg, pg)
    A_ag = AutogradOperator(A)
    x = torch.ones(A_ag.domain_shape, device=dev, requires_grad=True)
    y = A_ag(x)
    y.backward(y)
    assert torch.allclose(x.grad, A.T(A(x.detach())))
    p = torch.ones(A_ag.range_shape, device=dev, requires_grad=True)
    q = A_ag.T(p)
    q.backward(q)
    assert torch.allclose(p.grad, A(A.T(p.detach())))


@pytest.mark.parametrize("cone", [False, True])
def test_gradient_central_differences(dev, cone):
    """d/dx_i <w, A x> by central differences (eps = 1e-3) on 16 random voxels."""
    vg = ts.volume(shape=32, size=1)
    pg = (ts.cone(angles=40, shape=(32, 48), size=np.sqrt(2), cone_angle=0.5) if cone
          else ts.parallel(angles=40, shape=(32, 48), size=(1, 1.5)))
    A = ts.operator(vg, pg)
    f = to_autograd(A)
    gen = torch.Generator(device="cpu").manual_seed(4)
    x = torch.rand(A.domain_shape, generator=gen).to(dev).requires_grad_(True)
    w = torch.rand(A.range_shape, generator=gen).to(dev)
    (f(x) * w).sum().backward()
    idx = torch.randint(0, x.numel(), (16,), generator=gen)
    eps = 1e-3
    for i in idx.tolist():
        e = torch.zeros(x.numel(), device=dev)
        e[i] = eps
        e = e.view_as(x)
        lp = (A(x.detach() + e).double() * w.double()).sum()
        lm = (A(x.detach() - e).double() * w.double()).sum()
        fd = float((lp - lm) / (2 * eps))
        g = float(x.grad.view(-1)[i])
        assert fd == pytest.approx(g, rel=2e-2, abs=1e-4 * max(1.0, abs(g)))


def test_batched_extra_dims_equal_per_slice(dev):
    """to_autograd over (batch, channel) slices makes one batched C-ABI call
    (tsgb_direct_fp_batch / tsgb_direct_bp_batch) instead of a call per slice;
    the results equal projecting each slice on its own, bit for bit, forward
    and backward, for both matched backprojectors and for A.T as the operator."""
    vg = ts.volume(shape=(20, 24, 28), size=1)
    pg = ts.cone(angles=17, shape=(22, 30), size=(1.4, 1.6), cone_angle=0.4)
    A = ts.operator(vg, pg)
    for kernel in (0, 1):
        A.projector.set_tuning(dev.index, bp_kernel=kernel, bp_shape=0)
        f = to_autograd(A, num_extra_dims=2)
        x = torch.rand(2, 3, *A.domain_shape, device=dev, requires_grad=True)
        y = f(x)
        ref = torch.stack([torch.stack([A(x[i, j].detach()) for j in range(3)]) for i in range(2)])
        assert torch.equal(y, ref)
        g = torch.rand_like(y)
        y.backward(g)
        ref_g = torch.stack([torch.stack([A.T(g[i, j]) for j in range(3)]) for i in range(2)])
        assert torch.equal(x.grad, ref_g)
        fb = to_autograd(A.T, num_extra_dims=1)
        yy = torch.rand(4, *A.range_shape, device=dev)
        assert torch.equal(fb(yy), torch.stack([A.T(yy[i]) for i in range(4)]))


def test_batched_backprojection_in_groups_equals_per_item(dev):
    """A batched matched backprojection of the voxel-pair kernel runs on
    multi-job launches (one per pass over up to 48 items) when given the batch
    workspace: 50 items (two groups) equal backprojecting each on its own, bit
    for bit, setting and adding."""
    from tomosipo_gb300 import _native

    vg = ts.volume(shape=(16, 18, 20), size=1)
    pg = ts.cone(angles=9, shape=(16, 24), size=(1.2, 1.5), cone_angle=0.4)
    A = ts.operator(vg, pg)
    A.projector.set_tuning(dev.index, bp_kernel=0)
    lib = _native.load()
    h = A.projector.handle(dev.index)
    one = lib.tsgb_bp_workspace_bytes(h, 0)
    assert lib.tsgb_bp_batch_workspace_bytes(h, 50, 0) > one
    assert lib.tsgb_bp_batch_workspace_bytes(h, 1, 0) == one
    n = 50
    yy = torch.rand(n, *A.range_shape, device=dev)
    out = torch.full((n, *A.domain_shape), 7.0, device=dev)
    A.T._apply_batch(yy, out)
    ref = torch.stack([A.T(yy[i]) for i in range(n)])
    assert torch.equal(out, ref)
    B = ts.operator(vg, pg, additive=True)
    B.projector.set_tuning(dev.index, bp_kernel=0)
    acc = ref.clone()
    B.T._apply_batch(yy, acc)
    ref_add = ref.clone()
    for i in range(n):
        B.T(yy[i], out=ref_add[i])
    assert torch.equal(acc, ref_add)


def test_batched_forward_projection_in_groups_equals_per_item(dev):
    """A batched forward projection runs on multi-job launches (one ray launch
    over up to 48 items, each with its own volume copies) when given the batch
    workspace: 50 items equal projecting each on its own, bit for bit, setting
    and adding, for both copy layouts."""
    from tomosipo_gb300 import _native

    vg = ts.volume(shape=(16, 18, 20), size=1)
    pg = ts.cone(angles=9, shape=(16, 24), size=(1.2, 1.5), cone_angle=0.4)
    A = ts.operator(vg, pg)
    lib = _native.load()
    h = A.projector.handle(dev.index)
    assert lib.tsgb_fp_batch_workspace_bytes(h, 50) > lib.tsgb_fp_workspace_bytes(h)
    n = 50
    x = torch.rand(n, *A.domain_shape, device=dev)
    B = ts.operator(vg, pg, additive=True)
    for layout in (0, 1):
        for op in (A, B):
            op.projector.set_tuning(dev.index, fp_pair_layout=layout)
        out = torch.full((n, *A.range_shape), 3.0, device=dev)
        A._apply_batch(x, out)
        ref = torch.stack([A(x[i]) for i in range(n)])
        assert torch.equal(out, ref), layout
        acc = ref.clone()
        B._apply_batch(x, acc)
        ref_add = ref.clone()
        for i in range(n):
            B(x[i], out=ref_add[i])
        assert torch.equal(acc, ref_add), layout
