"""Small helpers for stacks of 3-vectors and 4x4 homogeneous matrices.

Covers the operations tomosipo's ``tomosipo/vector_calc.py`` provides to the
geometry classes: broadcasting of per-step vectors and matrices, dot and cross
products, ray/plane intersection and inversion of affine transforms.
Vectors are ``(N, 3)`` in ``(z, y, x)`` order; matrices are ``(N, 4, 4)``.
"""
import numpy as np

from . import types


def to_vec(x):
    """(N, 3) array; drops the homogeneous coordinate of an (N, 4) array."""
    x = np.array(x, dtype=np.float64, ndmin=2)
    if x.ndim == 2 and x.shape[1] == 4:
        return x[:, :3].copy()
    return types.to_vec(x)


def to_scalar(x):
    """(N, 1) array of scalars."""
    x = np.array(x, dtype=np.float64, ndmin=1)
    if x.ndim == 1:
        return x[:, None]
    if x.ndim == 2 and x.shape[1] == 1:
        return x
    raise ValueError(f"Expected scalar or (N,) array. Got shape {x.shape}.")


def to_homogeneous_vec(x):
    return types.to_homogeneous_vec(x)


def to_homogeneous_point(x):
    return types.to_homogeneous_pos(x)


def broadcast_lengths(len_a, len_b):
    if len_a == 1:
        return len_b
    if len_b == 1 or len_a == len_b:
        return len_a
    raise ValueError(f"Cannot broadcast lengths {len_a} and {len_b}.")


def _broadcastv(x, y):
    """Rows of vectors ``(N, k)`` (a single vector ``(k,)`` counts as one row),
    broadcast to a common number of rows; ``ValueError`` otherwise."""
    x, y = np.asarray(x), np.asarray(y)
    s1, s2 = x.shape, y.shape
    x, y = np.array(x, ndmin=2), np.array(y, ndmin=2)
    if x.ndim != 2 or y.ndim != 2 or x.shape[1] != y.shape[1]:
        raise ValueError(f"Arguments of shape {s1} and {s2} could not be broadcast together.")
    try:
        n = broadcast_lengths(len(x), len(y))
    except ValueError:
        raise ValueError(f"Arguments of shape {s1} and {s2} could not be broadcast together.")
    return np.broadcast_to(x, (n, x.shape[1])), np.broadcast_to(y, (n, y.shape[1]))


def _broadcastmv(m, x):
    """Matrices ``(N, a, b)`` (or one ``(a, b)``) and vectors ``(N, b)`` (or one
    ``(b,)``), broadcast to a common N."""
    m, x = np.asarray(m, dtype=np.float64), np.asarray(x, dtype=np.float64)
    s1, s2 = m.shape, x.shape
    m = m[None] if m.ndim == 2 else m
    x = x[None] if x.ndim == 1 else x
    if m.ndim != 3 or x.ndim != 2 or m.shape[2] != x.shape[1]:
        raise ValueError(f"Matrix of shape {s1} cannot transform vectors of shape {s2}.")
    try:
        n = broadcast_lengths(len(m), len(x))
    except ValueError:
        raise ValueError(f"Matrix of shape {s1} cannot transform vectors of shape {s2}.")
    return np.broadcast_to(m, (n,) + m.shape[1:]), np.broadcast_to(x, (n, x.shape[1]))


def _broadcastmm(m1, m2):
    """Two stacks of matrices ``(N, a, b)`` and ``(N, b, c)`` (single matrices
    count as one), broadcast to a common N."""
    m1, m2 = np.asarray(m1, dtype=np.float64), np.asarray(m2, dtype=np.float64)
    s1, s2 = m1.shape, m2.shape
    m1 = m1[None] if m1.ndim == 2 else m1
    m2 = m2[None] if m2.ndim == 2 else m2
    if m1.ndim != 3 or m2.ndim != 3 or m1.shape[2] != m2.shape[1]:
        raise ValueError(f"Matrices of shape {s1} and {s2} cannot be multiplied.")
    try:
        n = broadcast_lengths(len(m1), len(m2))
    except ValueError:
        raise ValueError(f"Matrices of shape {s1} and {s2} could not be broadcast together.")
    return np.broadcast_to(m1, (n,) + m1.shape[1:]), np.broadcast_to(m2, (n,) + m2.shape[1:])


def check_same_shapes(*args):
    shapes = [np.shape(a) for a in args]
    if min(shapes) != max(shapes):
        raise ValueError(f"Not all arguments are the same shape. Got: {shapes}")


def dot(x, y):
    x, y = _broadcastv(np.atleast_2d(x), np.atleast_2d(y))
    return np.einsum("ij,ij->i", x, y)


def squared_norm(x):
    return dot(x, x)


def norm(x):
    return np.sqrt(squared_norm(x))


def cross_product(x, y):
    """Cross product taken directly on the (z, y, x) components.

    This is the convention that fixes ``det_normal`` in tomosipo
    (``doc/topics/geometries.rst:364-410``: det_u = (0, 0, .1), det_v = (.1, 0, 0)
    gives det_normal = (0, .01, 0), pointing away from the source).
    """
    x, y = _broadcastv(np.atleast_2d(x), np.atleast_2d(y))
    return np.cross(x, y)


def intersect(v_origin, v_direction, plane_origin, plane_normal):
    """Point where each line ``origin + t * direction`` meets each plane.

    Lines parallel to their plane give NaN coordinates.
    """
    v_origin = to_vec(v_origin)
    v_direction = to_vec(v_direction)
    plane_origin = to_vec(plane_origin)
    plane_normal = to_vec(plane_normal)
    num = dot(plane_origin - v_origin, plane_normal)
    den = dot(v_direction, plane_normal)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = num / den
    t = np.where(np.abs(den) > 1e-300, t, np.nan)
    return v_origin + t[:, None] * v_direction


def matrix_transform(m, x):
    """Apply (N, a, b) matrices to (N, b) rows (broadcasting N): (N, a)."""
    m, x = _broadcastmv(m, x)
    return np.einsum("nij,nj->ni", m, x)


def matrix_matrix_transform(m1, m2):
    m1, m2 = _broadcastmm(m1, m2)
    return np.einsum("nij,njk->nik", m1, m2)


def invert_transformation_matrix(m):
    m = np.array(m, dtype=np.float64)
    if m.ndim == 2:
        m = m[None]
    return np.linalg.inv(m)
