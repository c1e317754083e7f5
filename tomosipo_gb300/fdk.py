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

dbeta_t is the source's angular step around the rotation axis through the
volume anchor (central differences of the unwrapped angles); the axis is the
mean direction of the detector's v axis, which FDK's setup keeps parallel to
it (z for ``ts.cone``). A full circle (2 pi) is the FDK case, and helical
scans are approximations as in any FDK. Short scans (``short_scan=True``:
pi plus the fan angle, up to a full circle) get Parker's redundancy weights
(D. L. Parker, Med. Phys. 9(2), 1982) before filtering, generalised to the
scan's own over-scan angle; the reference's ``accumulate_FDK`` call applies
none, so they are off by default. Steps 1 and 2 are torch element-wise ops
and a batched FFT on the device. Any cone geometry is accepted: angles whose
projection does not depend on z take the z-flat bilinear kernel, the others
(tilted detectors, rotated scans) the general bilinear kernel.
"""
import math

import numpy as np
import torch

from . import _native


def _vectors(pg):
    v = pg.to_vec()
    return tuple(np.asarray(a, dtype=np.float64) for a in (v.src_pos, v.det_pos, v.det_u, v.det_v))


def _anchor(vg):
    shape = np.array(vg.shape)
    return np.asarray(vg.lower_left_corner)[0] + (shape // 2 + 0.5) * np.asarray(vg.voxel_sizes)[0]


def rotation_frame(V):
    """Unit rotation axis (the mean direction of the detector v vectors) and
    two unit vectors e1, e2 spanning the plane normal to it, with
    e2 = axis x e1 (so angles atan2(r.e2, r.e1) grow counter-clockwise about
    the axis). For an axis along z, e1 is x."""
    axis = (V / np.linalg.norm(V, axis=1, keepdims=True)).mean(axis=0)
    axis /= np.linalg.norm(axis)
    # the coordinate axis least aligned with the rotation axis, orthogonalised
    e1 = np.eye(3)[[2, 1, 0][int(np.argmin(np.abs(axis[[2, 1, 0]])))]]
    e1 = e1 - np.dot(e1, axis) * axis
    e1 /= np.linalg.norm(e1)
    return axis, e1, np.cross(axis, e1)


def source_angles(S, anchor, V):
    """Unwrapped angle of each source position about the rotation axis through
    ``anchor``."""
    _, e1, e2 = rotation_frame(V)
    r = S - anchor[None]
    return np.unwrap(np.arctan2(r @ e2, r @ e1))


def fdk_constants(vg, pg):
    """Per-angle FDK constants (host, fp64): ``(sdd, pitch, angle_weight)``.

    ``sdd``: source to detector plane; ``pitch``: the filter's pixel pitch on
    the virtual detector through the anchor (the centre of voxel
    (nz/2, ny/2, nx/2), integer division, where the backprojector normalises
    depths); ``angle_weight``: dbeta / 2.
    """
    if not getattr(pg, "is_cone", False):
        raise ValueError("FDK reconstructs cone-beam geometries only")
    S, D, U, V = _vectors(pg)
    anchor = _anchor(vg)
    n = np.cross(U, V)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    n *= np.sign(np.einsum("ij,ij->i", D - S, n))[:, None]
    sdd = np.einsum("ij,ij->i", D - S, n)
    sod = np.einsum("ij,ij->i", anchor[None] - S, n)
    if np.any(sdd <= 0) or np.any(sod <= 0):
        raise ValueError("FDK needs the volume and the detector in front of the source")
    pitch = np.linalg.norm(U, axis=1) * sod / sdd
    beta = source_angles(S, anchor, V)
    dbeta = np.abs(np.gradient(beta)) if len(beta) > 1 else np.array([2 * math.pi])
    return sdd, pitch, dbeta / 2


def parker_weights(beta, gamma, delta):
    """Parker's redundancy weights for a short scan over [0, pi + 2 delta].

    ``beta``: source angle from the scan's start, in its direction of
    rotation; ``gamma``: fan angle of the ray, positive in the same direction
    (so the ray (beta, gamma) is measured again at (beta + pi + 2 gamma,
    -gamma)); ``delta`` >= max |gamma|: half the over-scan. The two weights of
    every such pair sum to 1. Arrays broadcast.
    """
    beta, gamma = np.asarray(beta, dtype=np.float64), np.asarray(gamma, dtype=np.float64)
    lo = 2 * (delta - gamma)  # end of the ramp-up
    hi = math.pi - 2 * gamma  # start of the ramp-down
    with np.errstate(divide="ignore", invalid="ignore"):
        up = np.sin(math.pi / 4 * beta / (delta - gamma)) ** 2
        down = np.sin(math.pi / 4 * (math.pi + 2 * delta - beta) / (delta + gamma)) ** 2
    w = np.where(beta < lo, up, np.where(beta <= hi, 1.0, down))
    return np.where((beta < 0) | (beta > math.pi + 2 * delta), 0.0, w)


def short_scan_weights(vg, pg):
    """Twice Parker's weights of every (angle, detector column), (angles, cols)
    fp64: a short scan measures each line once where a full circle measures it
    twice, and FDK's angle weight dbeta / 2 assumes the latter.

    The scan covers Delta = |beta_last - beta_first| + mean |dbeta|, centred
    on the source angles; delta = (Delta - pi) / 2 must cover the largest fan
    angle of the detector's columns (measured in the plane normal to the
    rotation axis)."""
    S, D, U, V = _vectors(pg)
    anchor = _anchor(vg)
    axis, _, _ = rotation_frame(V)
    beta = source_angles(S, anchor, V)
    n = len(beta)
    step = abs(beta[-1] - beta[0]) / (n - 1) if n > 1 else 2 * math.pi
    sign = 1.0 if n < 2 or beta[-1] >= beta[0] else -1.0
    coverage = abs(beta[-1] - beta[0]) + step
    delta = (coverage - math.pi) / 2
    cols = pg.det_shape[1]
    b = np.arange(cols) + 0.5 - cols / 2

    def perp(w):
        return w - (w @ axis)[..., None] * axis

    c = perp(anchor[None] - S)  # central ray (angles, 3)
    d = perp(D[:, None, :] + b[None, :, None] * U[:, None, :] - S[:, None, :])  # (angles, cols, 3)
    cross = np.cross(c[:, None, :], d) @ axis
    gamma = sign * np.arctan2(cross, np.einsum("ij,ikj->ik", c, d))
    if not delta >= np.abs(gamma).max():
        raise ValueError(
            "a short scan must cover pi plus the fan angle: {:.4f} rad covered, {:.4f} needed"
            .format(coverage, math.pi + 2 * np.abs(gamma).max()))
    rel = sign * (beta - beta[0]) + step / 2
    return 2 * parker_weights(rel[:, None], gamma, delta)


def fft_length(cols):
    """Smallest length >= 2 cols - 1 (a linear convolution of a row with the
    kernel's 2 cols - 1 taps, without wrap-around) whose prime factors are 2,
    3, 5 and 7 (fast FFT radices): 1536 for 768 columns, where the next power
    of two would be 2048."""
    n = max(2 * cols - 1, 2)
    while True:
        m = n
        for f in (2, 3, 5, 7):
            while m % f == 0:
                m //= f
        if m == 1 and n % 2 == 0:
            return n
        n += 1


def ramp_spectrum(cols, device):
    """Real spectrum of the unit-pitch Ram-Lak kernel, zero-padded to fft_length(cols)."""
    length = fft_length(cols)
    g = np.zeros(length)
    g[0] = 0.25
    odd = np.arange(1, cols, 2)
    g[odd] = -1.0 / (math.pi ** 2 * odd.astype(np.float64) ** 2)
    g[length - odd] = g[odd]
    return torch.from_numpy(np.fft.rfft(g).real.astype(np.float32)).to(device), length


def fdk_filter(vg, pg, y, angle_chunk=None, short_scan=False):
    """Cosine-weighted (and with ``short_scan`` Parker-weighted), ramp-filtered
    copy of sinogram ``y`` (a CUDA tensor). Angles are filtered ``angle_chunk``
    at a time (default: as many as fit a 512 MB zero-padded buffer)."""
    rows, nang, cols = y.shape
    dev = y.device
    if angle_chunk is None:
        angle_chunk = max(1, (512 << 20) // (rows * fft_length(cols) * 4))
    elif int(angle_chunk) < 1:
        raise ValueError(f"angle_chunk must be a positive number of angles, got {angle_chunk}")
    angle_chunk = int(angle_chunk)
    sdd, pitch, _ = fdk_constants(vg, pg)
    S, D, U, V = _vectors(pg)
    parker = (torch.from_numpy(short_scan_weights(vg, pg).astype(np.float32)).to(dev)
              if short_scan else None)
    w0 = D - S
    # |X - S|^2 = |w0 + a V + b U|^2 with a, b the pixel offsets from the centre
    per_angle = np.stack([
        np.einsum("ij,ij->i", w0, w0), np.einsum("ij,ij->i", V, V), np.einsum("ij,ij->i", U, U),
        2 * np.einsum("ij,ij->i", w0, V), 2 * np.einsum("ij,ij->i", w0, U),
        2 * np.einsum("ij,ij->i", U, V), sdd, 1.0 / pitch,
    ], axis=1)
    # A circular scan (the detector turning with the source) has the same
    # cosine-weight coefficients (the first 7) at every angle: one weight map
    # then serves all angles. (Compared relative to the largest: some are zero
    # up to rounding. The last, 1 / pitch, can vary: the pitch is referred to
    # the anchor voxel, off the rotation axis by half a voxel in an even-sized
    # volume; it is applied per angle either way.)
    cw = per_angle[:, :7]
    same = bool(np.all(np.abs(cw - cw[:1]) <= 1e-12 * np.abs(cw).max()))
    c = torch.from_numpy(per_angle).to(dev)
    a = torch.arange(rows, device=dev, dtype=torch.float64) + 0.5 - rows / 2
    b = torch.arange(cols, device=dev, dtype=torch.float64) + 0.5 - cols / 2

    def cosine_weights(k):
        A, B = a[:, None, None], b[None, None, :]
        dist2 = (k[None, :, 0, None] + A * A * k[None, :, 1, None] + B * B * k[None, :, 2, None]
                 + A * k[None, :, 3, None] + B * k[None, :, 4, None] + A * B * k[None, :, 5, None])
        return (k[None, :, 6, None] / torch.sqrt(dist2)).to(torch.float32)

    shared = cosine_weights(c[:1]) if same else None
    spec, length = ramp_spectrum(cols, dev)
    q = torch.empty_like(y, dtype=torch.float32)
    buf = None  # weighted rows, zero-padded to the FFT length (the padding stays zero)
    for t0 in range(0, nang, angle_chunk):
        t1 = min(nang, t0 + angle_chunk)
        if buf is None or buf.shape[1] != t1 - t0:
            buf = torch.zeros((rows, t1 - t0, length), dtype=torch.float32, device=dev)
        k = c[t0:t1]
        w = shared if same else cosine_weights(k)
        if parker is not None:
            w = w * parker[None, t0:t1, :]
        torch.mul(y[:, t0:t1, :].to(torch.float32), w, out=buf[..., :cols])
        f = torch.fft.rfft(buf, dim=-1)
        # the ramp times each angle's 1 / pitch, in one pass over the spectrum
        f.mul_(spec * k[None, :, 7, None].to(torch.float32))
        q[:, t0:t1, :] = torch.fft.irfft(f, n=length, dim=-1)[..., :cols]
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


def fdk_reconstruct(vg, pg, y, out=None, additive=False, projector=None, short_scan=False):
    """FDK reconstruction of sinogram ``y`` (CUDA tensor, (rows, angles, cols)).

    Returns ``out`` (a CUDA volume tensor, created if None; added to when
    ``additive``). ``short_scan``: apply Parker's redundancy weights (scans of
    pi plus the fan angle or more, less than a full circle).
    """
    from .projector import create_projector

    if not (isinstance(y, torch.Tensor) and y.is_cuda):
        raise ValueError("fdk_reconstruct expects a CUDA tensor sinogram")
    projector = projector or create_projector(vg, pg)
    q = fdk_filter(vg, pg, y, short_scan=short_scan)
    if out is None:
        out = torch.zeros(tuple(vg.shape), dtype=torch.float32, device=y.device)
        additive = True
    fdk_backproject(projector, out, q, fdk_constants(vg, pg)[2], additive)
    return out
