"""Shared test inputs: seeded phantoms and the geometries the parity tests use."""
import numpy as np

import tomosipo_gb300 as ts

# Accuracy gates. fp32 kernels vs the FP64 oracle: relative L2 error.
TOL_ORACLE = 1e-5
# |<Ax, y> - <x, A^T y>| / (|Ax| |y|), dot products in float64.
TOL_ADJOINT = 1e-6


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def adjoint_error(Ax, y, x, ATy):
    lhs = float(np.dot(np.asarray(Ax, np.float64).ravel(), np.asarray(y, np.float64).ravel()))
    rhs = float(np.dot(np.asarray(x, np.float64).ravel(), np.asarray(ATy, np.float64).ravel()))
    return abs(lhs - rhs) / (np.linalg.norm(np.asarray(Ax, np.float64)) * np.linalg.norm(np.asarray(y, np.float64)))


def noise_cube_phantom(shape, seed=0):
    """Uniform [0, 1) noise plus a unit cube on voxels [20:50]^3 (scaled to shape)."""
    rng = np.random.default_rng(seed)
    x = rng.random(shape)
    lo = [int(round(20 / 64 * n)) for n in shape]
    hi = [int(round(50 / 64 * n)) for n in shape]
    x[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += 1.0
    return x.astype(np.float32)


def ellipsoid_phantom(shape, n=20, seed=1):
    """Sum of ``n`` random ellipsoids with densities U[0.1, 1] on [-1, 1]^3."""
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.meshgrid(*[np.linspace(-1, 1, s) for s in shape], indexing="ij")
    x = np.zeros(shape, dtype=np.float32)
    for _ in range(n):
        c = rng.uniform(-0.5, 0.5, 3)
        r = rng.uniform(0.1, 0.45, 3)
        rho = rng.uniform(0.1, 1.0)
        m = ((zz - c[0]) / r[0]) ** 2 + ((yy - c[1]) / r[1]) ** 2 + ((xx - c[2]) / r[2]) ** 2 <= 1
        x[m] += rho
    return x


def helical_cone_vec(num_angles, shape, size, src_dist, det_dist, pitch, turns=1.0,
                     jitter=0.0, voxel=1.0, seed=5):
    """Helical cone_vec: source and detector turn ``turns`` times around z and rise
    by ``pitch`` per turn (centred on z = 0).

    ``jitter`` is the standard deviation, in units of ``voxel``, of independent
    per-angle source and detector position noise. det_v stays along z.
    """
    rng = np.random.default_rng(seed)
    t = np.linspace(0, 2 * np.pi * turns, num_angles, endpoint=False)
    rise = pitch * (t / (2 * np.pi) - turns / 2)
    c, s = np.cos(t), np.sin(t)
    src = np.stack([rise, -c * src_dist, s * src_dist], axis=1)
    det = np.stack([rise, c * det_dist, -s * det_dist], axis=1)
    if jitter:
        src = src + rng.normal(0, jitter * voxel, src.shape)
        det = det + rng.normal(0, jitter * voxel, det.shape)
    sv = size[0] / shape[0]
    su = size[1] / shape[1]
    det_v = np.stack([np.full_like(t, sv), 0 * t, 0 * t], axis=1)
    det_u = np.stack([0 * t, s * su, c * su], axis=1)
    return ts.cone_vec(shape=shape, src_pos=src, det_pos=det, det_v=det_v, det_u=det_u)
