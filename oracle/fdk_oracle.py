"""FP64 NumPy FDK -- TEST INFRASTRUCTURE ONLY.

The oracle for ``tomosipo_gb300.fdk`` (tomosipo's ``fdk``,
``tomosipo/astra.py:374-406``), written independently of it: world-space
ray/plane intersections instead of the kernels' projection matrices, and the
ramp filter as a direct spatial convolution instead of an FFT. The method is
Feldkamp, Davis & Kress (J. Opt. Soc. Am. A 1(6), 1984) for flat detectors:
cosine weights SDD / |X - S|; the Ram-Lak filter h[0] = 1/(4 d^2),
h[odd n] = -1/(pi^2 n^2 d^2) on the virtual detector through the reference
point (pitch d = |det_u| SOD / SDD), applied as d * sum_n h[k - n] p[n]; and
the backprojection sum_t (dbeta_t / 2) (SOD_t / U_t(x))^2 q_t(u, v) with
bilinear detector reads (zero outside the detector). The reference point is
the centre of voxel (nz/2, ny/2, nx/2), integer division; dbeta_t are
central differences of the source's unwrapped angle around the rotation axis
(the normalised mean of the detector's unit v vectors) through it. Short
scans: Parker's weights (Med. Phys. 9(2), 1982) with the over-scan half-angle
delta = (coverage - pi) / 2, times 2, on the cosine-weighted data.
Small cases only (pure NumPy).
"""
import math

import numpy as np


def _frame(vg, pg):
    v = pg.to_vec()
    S, D, U, V = (np.asarray(a, dtype=np.float64) for a in (v.src_pos, v.det_pos, v.det_u, v.det_v))
    shape = np.array(vg.shape)
    vs = np.asarray(vg.voxel_sizes, dtype=np.float64).reshape(3)
    llc = np.asarray(vg.lower_left_corner, dtype=np.float64).reshape(3)
    ref = llc + (shape // 2 + 0.5) * vs
    return S, D, U, V, shape, vs, llc, ref


def _normal_depths(S, D, U, V, ref, t):
    """Unit detector normal pointing away from the source, SDD and SOD of angle t."""
    n = np.cross(U[t], V[t])
    n /= np.linalg.norm(n)
    if np.dot(D[t] - S[t], n) < 0:
        n = -n
    return n, np.dot(D[t] - S[t], n), np.dot(ref - S[t], n)


def _axis_angles(S, V, ref):
    """Rotation axis and the unwrapped source angles about it (counter-clockwise
    about the axis, from an arbitrary in-plane direction)."""
    axis = sum(v / np.linalg.norm(v) for v in V)
    axis = axis / np.linalg.norm(axis)
    # in-plane basis: Gram-Schmidt of the world axis least parallel to the axis
    k = int(np.argmin(np.abs(axis)))
    p = np.zeros(3)
    p[k] = 1.0
    p -= (p @ axis) * axis
    p /= np.linalg.norm(p)
    q = np.cross(axis, p)
    ang = [math.atan2((s - ref) @ q, (s - ref) @ p) for s in S]
    return axis, np.unwrap(ang)


def angle_weights(vg, pg):
    """dbeta_t / 2: half the source's angular step around the rotation axis
    through the reference point (central differences of the unwrapped angle)."""
    S, _, _, V, _, _, _, ref = _frame(vg, pg)
    _, beta = _axis_angles(S, V, ref)
    return (np.abs(np.gradient(beta)) if len(S) > 1 else np.array([2 * math.pi])) / 2


def parker(vg, pg):
    """2 x Parker's weight of each (angle, column) of a short scan."""
    S, D, U, V, _, _, _, ref = _frame(vg, pg)
    axis, beta = _axis_angles(S, V, ref)
    N = len(S)
    C = pg.det_shape[1]
    step = abs(beta[-1] - beta[0]) / (N - 1)
    direction = 1.0 if beta[-1] > beta[0] else -1.0
    delta = (abs(beta[-1] - beta[0]) + step - math.pi) / 2
    w = np.zeros((N, C))
    for t in range(N):
        b = direction * (beta[t] - beta[0]) + step / 2
        c = ref - S[t]
        c = c - (c @ axis) * axis
        for j in range(C):
            d = D[t] + (j + 0.5 - C / 2) * U[t] - S[t]
            d = d - (d @ axis) * axis
            g = direction * math.atan2(np.cross(c, d) @ axis, c @ d)
            assert abs(g) <= delta, "scan shorter than pi plus the fan angle"
            if b < 2 * (delta - g):
                w[t, j] = math.sin(math.pi / 4 * b / (delta - g)) ** 2
            elif b <= math.pi - 2 * g:
                w[t, j] = 1.0
            elif b <= math.pi + 2 * delta:
                w[t, j] = math.sin(math.pi / 4 * (math.pi + 2 * delta - b) / (delta + g)) ** 2
    return 2 * w


def filtered(vg, pg, y, short_scan=False):
    """Cosine-weighted, ramp-filtered sinogram (fp64, (rows, angles, cols)): steps
    1 and 2 of FDK, with the Ram-Lak filter as a direct convolution."""
    S, D, U, V, _, _, _, ref = _frame(vg, pg)
    pw = parker(vg, pg) if short_scan else None
    y = np.asarray(y, dtype=np.float64)
    R, N, C = y.shape
    k = np.arange(-(C - 1), C)
    h1 = np.zeros(k.shape)  # unit-pitch Ram-Lak kernel, k = -(C-1) .. C-1
    h1[k == 0] = 0.25
    odd = k % 2 != 0
    h1[odd] = -1.0 / (math.pi ** 2 * k[odd].astype(np.float64) ** 2)
    a = np.arange(R) + 0.5 - R / 2
    b = np.arange(C) + 0.5 - C / 2
    q = np.empty_like(y)
    for t in range(N):
        _, sdd, sod = _normal_depths(S, D, U, V, ref, t)
        d = np.linalg.norm(U[t]) * sod / sdd
        X = D[t] + a[:, None, None] * V[t] + b[None, :, None] * U[t]
        p = y[:, t, :] * sdd / np.linalg.norm(X - S[t], axis=-1)
        if pw is not None:
            p = p * pw[t][None, :]
        q[:, t, :] = np.stack([np.convolve(p[r], h1)[C - 1:2 * C - 1] for r in range(R)]) / d
    return q


def fdk(vg, pg, y, short_scan=False):
    """FDK reconstruction (fp64 volume) of sinogram ``y`` ((rows, angles, cols))."""
    S, D, U, V, shape, vs, llc, ref = _frame(vg, pg)
    R, N, C = np.shape(y)
    # voxel centres (world)
    grids = [llc[i] + (np.arange(shape[i]) + 0.5) * vs[i] for i in range(3)]
    P = np.stack(np.meshgrid(*grids, indexing="ij"), axis=-1).reshape(-1, 3)
    out = np.zeros(P.shape[0])
    half_dbeta = angle_weights(vg, pg)
    Q = filtered(vg, pg, y, short_scan)
    for t in range(N):
        n, sdd, sod = _normal_depths(S, D, U, V, ref, t)
        q = Q[:, t, :]
        # project voxel centres: ray S -> P meets the detector plane at X
        rel = P - S[t]
        depth = rel @ n
        Xp = S[t] + rel * (sdd / depth)[:, None]
        G = np.array([[U[t] @ U[t], U[t] @ V[t]], [U[t] @ V[t], V[t] @ V[t]]])
        rhs = np.stack([(Xp - D[t]) @ U[t], (Xp - D[t]) @ V[t]], axis=1)
        uv = np.linalg.solve(G, rhs.T).T  # pixel offsets from the detector centre
        u = uv[:, 0] + C / 2 - 0.5
        v = uv[:, 1] + R / 2 - 0.5
        i0, j0 = np.floor(v).astype(int), np.floor(u).astype(int)
        fi, fj = v - i0, u - j0
        val = np.zeros(P.shape[0])
        for di, wi in ((0, 1 - fi), (1, fi)):
            for dj, wj in ((0, 1 - fj), (1, fj)):
                ii, jj = i0 + di, j0 + dj
                ok = (ii >= 0) & (ii < R) & (jj >= 0) & (jj < C)
                val[ok] += (wi * wj)[ok] * q[ii[ok], jj[ok]]
        out += half_dbeta[t] * (sod / depth) ** 2 * val
    return out.reshape(tuple(shape))
