"""FDK reconstruction for cone beams (tomosipo's ``fdk``, ``tomosipo/astra.py:374-406``).

The reference hands this to ASTRA's ``accumulate_FDK``. Here it is the
Feldkamp-Davis-Kress method for flat detectors (J. Opt. Soc. Am. A 1(6),
1984), with the backprojection on this package's GPU kernel:

1. weight every pixel by the cosine of its ray's angle to the detector
   normal, ``SDD / |X - S|`` (S source, X pixel centre, SDD the source's
   distance to the detector plane);
2. filter every detector row with the ramp (Ram-Lak) filter sampled on the
   virtual detector through the volume anchor, whose pixel pitch is
   ``|det_u| * SOD / SDD`` (SOD the anchor's depth along the detector normal):
   h[0] = 1 / (4 d^2), h[n] = -1 / (pi^2 n^2 d^2) for odd n, 0 for even n,
   as a zero-padded FFT convolution times d;
3. backproject ``sum_t (dbeta_t / 2) (SOD / U_t(x))^2 q_t(u_t(x), v_t(x))``
   (U_t(x) the voxel's depth along the normal) with bilinear detector reads:
   ``tsgb_fdk_backproject``.

dbeta_t is the source's angular step around the z axis through the volume
anchor (central differences of the unwrapped angles). A full circle (2 pi)
is the FDK case; shorter scans would need redundancy (Parker) weights, which
are not applied, and helical scans are approximations as in any FDK.
Steps 1 and 2 are torch element-wise ops and a batched FFT on the device.
Cone beams whose detector v axis runs along z are supported (circular and
helical ``cone``/``cone_vec``); other geometries raise ``ValueError``.
"""
import math

import numpy as np
import torch

from . import _native


def fdk_constants(vg, pg):
    """Per-angle FDK constants (host, fp64): ``(sdd, pitch, angle_weight)``.

    ``sdd``: source to detector plane; ``pitch``: the filter's pixel pitch on
    the virtual detector through the anchor (the centre of voxel
    (nz/2, ny/2, nx/2), integer division, where the backprojector normalises
    depths); ``angle_weight``: dbeta / 2.
    """
    if not getattr(pg, "is_cone", False):
        raise ValueError("FDK reconstructs cone-beam geometries only")
    v = pg.to_vec()
    S, D, U, V = (np.asarray(a, dtype=np.float64) for a in (v.src_pos, v.det_pos, v.det_u, v.det_v))
    shape = np.array(vg.shape)
    anchor = np.asarray(vg.lower_left_corner)[0] + (shape // 2 + 0.5) * np.asarray(vg.voxel_sizes)[0]
    n = np.cross(U, V)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    n *= np.sign(np.einsum("ij,ij->i", D - S, n))[:, None]
    sdd = np.einsum("ij,ij->i", D - S, n)
    sod = np.einsum("ij,ij->i", anchor[None] - S, n)
    if np.any(sdd <= 0) or np.any(sod <= 0):
        raise ValueError("FDK needs the volume and the detector in front of the source")
    pitch = np.linalg.norm(U, axis=1) * sod / sdd
    beta = np.unwrap(np.arctan2(S[:, 1] - anchor[1], S[:, 2] - anchor[2]))
    dbeta = np.abs(np.gradient(beta)) if len(beta) > 1 else np.array([2 * math.pi])
    return sdd, pitch, dbeta / 2


def ramp_spectrum(cols, device):
    """Real spectrum of the unit-pitch Ram-Lak kernel, zero-padded to >= 2 cols."""
    length = 1 << int(math.ceil(math.log2(max(2 * cols, 2))))
    g = np.zeros(length)
    g[0] = 0.25
    odd = np.arange(1, cols, 2)
    g[odd] = -1.0 / (math.pi ** 2 * odd.astype(np.float64) ** 2)
    g[length - odd] = g[odd]
    return torch.from_numpy(np.fft.rfft(g).real.astype(np.float32)).to(device), length


def fdk_filter(vg, pg, y, angle_chunk=64):
    """Cosine-weighted, ramp-filtered copy of sinogram ``y`` (a CUDA tensor)."""
    rows, nang, cols = y.shape
    dev = y.device
    sdd, pitch, _ = fdk_constants(vg, pg)
    v = pg.to_vec()
    S, D, U, V = (np.asarray(a, dtype=np.float64) for a in (v.src_pos, v.det_pos, v.det_u, v.det_v))
    w0 = D - S
    # |X - S|^2 = |w0 + a V + b U|^2 with a, b the pixel offsets from the centre
    per_angle = np.stack([
        np.einsum("ij,ij->i", w0, w0), np.einsum("ij,ij->i", V, V), np.einsum("ij,ij->i", U, U),
        2 * np.einsum("ij,ij->i", w0, V), 2 * np.einsum("ij,ij->i", w0, U),
        2 * np.einsum("ij,ij->i", U, V), sdd, 1.0 / pitch,
    ], axis=1)
    c = torch.from_numpy(per_angle).to(dev)
    a = torch.arange(rows, device=dev, dtype=torch.float64) + 0.5 - rows / 2
    b = torch.arange(cols, device=dev, dtype=torch.float64) + 0.5 - cols / 2
    spec, length = ramp_spectrum(cols, dev)
    q = torch.empty_like(y, dtype=torch.float32)
    for t0 in range(0, nang, angle_chunk):
        t1 = min(nang, t0 + angle_chunk)
        k = c[t0:t1]
        A, B = a[:, None, None], b[None, None, :]
        dist2 = (k[None, :, 0, None] + A * A * k[None, :, 1, None] + B * B * k[None, :, 2, None]
                 + A * k[None, :, 3, None] + B * k[None, :, 4, None] + A * B * k[None, :, 5, None])
        cosw = (k[None, :, 6, None] / torch.sqrt(dist2)).to(torch.float32)
        p = y[:, t0:t1, :].to(torch.float32) * cosw
        f = torch.fft.irfft(torch.fft.rfft(p, n=length, dim=-1) * spec, n=length, dim=-1)[..., :cols]
        q[:, t0:t1, :] = f * k[None, :, 7, None].to(torch.float32)
    return q


def fdk_backproject(projector, vol, q, angle_weight, additive):
    """``vol (+)= sum_t angle_weight[t] (SOD / U)^2 q_t(u, v)`` on the GPU."""
    lib = _native.load()
    dev = vol.device
    with torch.cuda.device(dev):
        h = projector.handle(dev.index)
        w = torch.as_tensor(np.asarray(angle_weight, dtype=np.float32), device=dev)
        nbytes = projector.workspace_bytes(dev.index, False, "bilinear")
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _native.check(lib.tsgb_fdk_backproject(h, vol.data_ptr(), q.data_ptr(), w.data_ptr(),
                                               int(bool(additive)), ws.data_ptr(), nbytes, stream),
                      "tsgb_fdk_backproject")


def fdk_reconstruct(vg, pg, y, out=None, additive=False, projector=None):
    """FDK reconstruction of sinogram ``y`` (CUDA tensor, (rows, angles, cols)).

    Returns ``out`` (a CUDA volume tensor, created if None; added to when
    ``additive``).
    """
    from .projector import create_projector

    if not (isinstance(y, torch.Tensor) and y.is_cuda):
        raise ValueError("fdk_reconstruct expects a CUDA tensor sinogram")
    projector = projector or create_projector(vg, pg)
    q = fdk_filter(vg, pg, y)
    if out is None:
        out = torch.zeros(tuple(vg.shape), dtype=torch.float32, device=y.device)
        additive = True
    fdk_backproject(projector, out, q, fdk_constants(vg, pg)[2], additive)
    return out
