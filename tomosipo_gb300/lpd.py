"""Unrolled learned primal-dual reconstruction on the GB300 projector.

Follows the structure of the reference's ``notebooks/learned_pd.py:48-99``
(Adler & Oktem's learned primal-dual with ReLU and no biases): ``n_iters``
unrolled iterations, a dual memory of 5 sinogram-shaped channels updated from
(h, A f, g) and a primal memory of 5 volume-shaped channels updated from
(f, A^T h). Here the network is 3-D: every block is three 3x3x3 convolutions
with ``channels`` hidden channels, on volumes and on sinograms (rows, angles,
cols) alike. The projector runs in fp32 through ``to_autograd`` (backward =
the matched backprojection, the exact adjoint); the convolutions run in
``dtype`` (bf16 by default, Kaiming-initialised weights) on channels-last
(NDHWC) tensors, which cuDNN's 3-D convolutions run about 1.5x faster than
NCDHW at 32 channels. With ``checkpoint=True`` each iteration is recomputed in
the backward pass instead of storing its activations.

(The reference's closures ``fp``/``bp`` call undefined names ``op``/``opT``,
``learned_pd.py:81-88``; here they call the module's own operators.)
"""
import torch
import torch.nn as nn
from torch.utils.checkpoint import checkpoint as _checkpoint

from .torch_support import to_autograd


def _activation(name):
    if name == "relu":
        return nn.ReLU()
    if name == "softplus":  # smooth stand-in, used for tight finite-difference checks
        return nn.Softplus(beta=10)
    raise ValueError(f"unknown activation {name!r}")


def _block(cin, channels, cout, dtype, activation="relu"):
    layers = [
        nn.Conv3d(cin, channels, kernel_size=3, padding=1, bias=False),
        _activation(activation),
        nn.Conv3d(channels, channels, kernel_size=3, padding=1, bias=False),
        _activation(activation),
        nn.Conv3d(channels, cout, kernel_size=3, padding=1, bias=False),
    ]
    for m in layers:
        if isinstance(m, nn.Conv3d):
            nn.init.kaiming_normal_(m.weight, nonlinearity="relu")
    return nn.Sequential(*layers).to(dtype=dtype, memory_format=torch.channels_last_3d)


class LearnedPrimalDual3d(nn.Module):
    """Learned primal-dual with a 3-D CNN per unrolled iteration.

    Input ``g``: (batch, 1, rows, angles, cols) fp32 sinograms. Output: (batch,
    1, z, y, x) fp32 reconstructions. ``f0`` optionally gives the initial
    primal estimate (batch, 1, z, y, x).
    """

    def __init__(self, A, n_iters=10, channels=32, dtype=torch.bfloat16, checkpoint=True,
                 activation="relu"):
        super().__init__()
        self.A = A
        self.n_iters = n_iters
        self.dtype = dtype
        self.use_checkpoint = checkpoint
        self.fp = to_autograd(A, num_extra_dims=2)
        self.bp = to_autograd(A.T, num_extra_dims=2)
        self.primal = nn.ModuleList(
            [_block(6, channels, 5, dtype, activation) for _ in range(n_iters)])
        self.dual = nn.ModuleList(
            [_block(7, channels, 5, dtype, activation) for _ in range(n_iters)])

    def _iteration(self, i, g, h, f):
        cl = torch.channels_last_3d
        f_dual = self.fp(f[:, :1])
        x = torch.cat((h, f_dual, g), dim=1).to(self.dtype, memory_format=cl)
        h = h + self.dual[i](x).float()
        update = self.bp(h[:, :1])
        x = torch.cat((f, update), dim=1).to(self.dtype, memory_format=cl)
        f = f + self.primal[i](x).float()
        return h, f

    def forward(self, g, f0=None):
        B = g.shape[0]
        h = g.new_zeros(B, 5, *g.shape[2:])
        f = g.new_zeros(B, 5, *self.A.domain_shape)
        if f0 is not None:
            f = torch.cat((f0, f[:, 1:]), dim=1)
        for i in range(self.n_iters):
            if self.use_checkpoint and torch.is_grad_enabled():
                h, f = _checkpoint(self._iteration, i, g, h, f, use_reentrant=False)
            else:
                h, f = self._iteration(i, g, h, f)
        return f[:, :1]
