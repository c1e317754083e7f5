"""Affine transforms of geometries (time-dependent 4x4 homogeneous matrices).

Same API and conventions as tomosipo's ``tomosipo/geometry/transform.py``:
``translate``, ``scale``, ``rotate``, ``reflect``, ``to_perspective``,
``from_perspective``. Coordinates are ``(z, y, x)``; ``rotate`` is right-handed
in the physical (x, y, z) frame by default. A transform with one step
broadcasts against geometries and transforms with many steps.
"""
import warnings

import numpy as np

from .. import types
from .. import vector_calc as vc

EPSILON = 1e-8


class Transform:
    """A stack of ``num_steps`` affine transforms, shape ``(num_steps, 4, 4)``."""

    def __init__(self, matrix):
        m = np.array(matrix, dtype=np.float64)
        if m.ndim == 2:
            m = m[None]
        if m.ndim != 3 or m.shape[1:] != (4, 4):
            raise ValueError(f"Expected (N, 4, 4) matrix. Got shape {m.shape}.")
        self.matrix = m

    def __mul__(self, other):
        if isinstance(other, Transform):
            if not (
                self.num_steps == 1
                or other.num_steps == 1
                or self.num_steps == other.num_steps
            ):
                raise ValueError(
                    "Cannot multiply transforms with different number of time steps. "
                    f"Got steps: {self.num_steps} and {other.num_steps}"
                )
            return Transform(vc.matrix_matrix_transform(self.matrix, other.matrix))
        return NotImplemented

    def __repr__(self):
        return f"Transform(\n    {self.matrix}\n)"

    def __eq__(self, other):
        if not isinstance(other, Transform):
            return False
        try:
            a, b = vc._broadcastmm(self.matrix, other.matrix)
        except ValueError:
            return False
        return bool(np.all(np.abs(a - b) < EPSILON))

    def __getitem__(self, i):
        if not isinstance(i, (slice, int, np.integer)):
            raise TypeError(f"Transform only support one-dimensional indexing. Got: {i}")
        return Transform(self.matrix[i])

    def __len__(self):
        return self.num_steps

    @property
    def num_steps(self):
        return self.matrix.shape[0]

    @property
    def inv(self):
        return Transform(vc.invert_transformation_matrix(self.matrix))

    def transform_vec(self, vec):
        """Apply to direction vectors (no translation); returns (N, 3)."""
        return vc.to_vec(vc.matrix_transform(self.matrix, vc.to_homogeneous_vec(vec)))

    def transform_point(self, points):
        """Apply to points (with translation); returns (N, 3)."""
        return vc.to_vec(
            vc.matrix_transform(self.matrix, vc.to_homogeneous_point(points))
        )


def identity():
    return Transform(np.eye(4))


def translate(axis, *, alpha=1):
    """Translation by ``alpha * axis`` (``axis`` may hold one row per step)."""
    axis = vc.to_homogeneous_point(axis)
    alpha = types.to_scalars(alpha, var_name="alpha")
    if not (len(axis) == 1 or len(alpha) == 1 or len(axis) == len(alpha)):
        raise ValueError(
            "Expected parameters `axis` and `alpha` to be the same length. "
            f"Got: {len(axis)}, {len(alpha)}"
        )
    t = alpha[:, None] * axis[:, :3]
    m = np.broadcast_to(np.eye(4), (len(t), 4, 4)).copy()
    m[:, :3, 3] = t
    return Transform(m)


def scale(scale, *, pos=0, alpha=1.0):
    """Scaling by ``alpha * scale`` around ``pos``."""
    if np.isscalar(scale):
        scale = types.to_size3d(scale)
    if np.isscalar(pos):
        pos = types.to_pos(pos)
    s = types.to_homogeneous_vec(scale)[:, :3]
    p = types.to_homogeneous_pos(pos)
    alpha = types.to_scalars(alpha)
    l1, l2, l3 = len(s), len(p), len(alpha)
    try:
        n = vc.broadcast_lengths(vc.broadcast_lengths(l1, l2), l3)
    except ValueError:
        raise ValueError(
            "Expected `scale`, `pos`, and `alpha` to be broadcastable. "
            f"Got lengths: {l1}, {l2}, and {l3}."
        )
    s = np.broadcast_to(alpha[:, None] * s, (n, 3))
    m = np.zeros((n, 4, 4))
    m[:, 0, 0], m[:, 1, 1], m[:, 2, 2] = s[:, 0], s[:, 1], s[:, 2]
    m[:, 3, 3] = 1.0
    T = translate(p)
    return T * Transform(m) * T.inv


def rotate(*, pos, axis, angles=None, rad=None, deg=None, right_handed=True):
    """Rotation by ``angles`` (radians) around ``axis`` through ``pos``.

    In (z, y, x) component order the right-handed Rodrigues matrix is
    ``cos(t) I - sin(t) [a]_x + (1 - cos(t)) a a^T``: reversing the three axes
    flips the sign of the cross-product matrix.
    """
    if np.isscalar(pos):
        pos = types.to_pos(pos)
    p = vc.to_homogeneous_point(pos)
    a = vc.to_homogeneous_vec(axis)
    p, a = vc._broadcastv(p, a)
    a = a[:, :3] / vc.norm(a[:, :3])[:, None]

    if angles is None and rad is None and deg is None:
        raise ValueError("The `angles=` parameter is required.")
    if angles is not None and (rad is not None or deg is not None):
        raise TypeError(
            "The `angles` parameter is not compatible with the `rad` or `deg` parameter. "
            "The `rad` and `deg` parameters are deprecated. "
        )
    if angles is None:
        warnings.warn(
            "The `rad` and `deg` parameters of `ts.rotate` are deprecated. "
            "Please use `angles` instead.",
            category=DeprecationWarning,
            stacklevel=2,
        )
        angles = np.deg2rad(deg) if deg is not None else rad
    theta = vc.to_scalar(angles)[:, 0]
    if not right_handed:
        theta = -theta

    n = vc.broadcast_lengths(len(a), len(theta))
    a = np.broadcast_to(a, (n, 3))
    theta = np.broadcast_to(theta, (n,))
    c, s = np.cos(theta), np.sin(theta)
    cross = np.zeros((n, 3, 3))
    cross[:, 0, 1], cross[:, 0, 2] = -a[:, 2], a[:, 1]
    cross[:, 1, 0], cross[:, 1, 2] = a[:, 2], -a[:, 0]
    cross[:, 2, 0], cross[:, 2, 1] = -a[:, 1], a[:, 0]
    r3 = (
        c[:, None, None] * np.eye(3)
        - s[:, None, None] * cross
        + (1 - c)[:, None, None] * np.einsum("ni,nj->nij", a, a)
    )
    m = np.zeros((n, 4, 4))
    m[:, :3, :3] = r3
    m[:, 3, 3] = 1.0
    T = translate(p)
    return T * Transform(m) * T.inv


def reflect(*, pos, axis):
    """Reflection in the plane through ``pos`` with normal ``axis``."""
    if np.isscalar(pos):
        pos = types.to_pos(pos)
    p = vc.to_homogeneous_point(pos)
    a = vc.to_homogeneous_vec(axis)
    p, a = vc._broadcastv(p, a)
    a = a[:, :3] / vc.norm(a[:, :3])[:, None]
    m = np.broadcast_to(np.eye(4), (len(a), 4, 4)).copy()
    m[:, :3, :3] -= 2 * np.einsum("ni,nj->nij", a, a)
    T = translate(p)
    return T * Transform(m) * T.inv


def to_perspective(*, pos=None, w=None, v=None, u=None, vol=None, ignore_scale=True):
    """Transform from the frame ``(pos; w, v, u)`` to world coordinates."""
    if vol is not None:
        pos, w, v, u = vol.pos, vol.w, vol.v, vol.u
    if any(x is None for x in (pos, w, v, u)):
        raise ValueError("Not enough arguments provided: one of pos, w, v, u is missing.")
    pos = vc.to_homogeneous_point(pos)
    w, v, u = (vc.to_homogeneous_vec(x) for x in (w, v, u))
    pos, w, v, u = np.broadcast_arrays(pos, w, v, u)
    if ignore_scale:
        w = w / vc.norm(w[:, :3])[:, None]
        v = v / vc.norm(v[:, :3])[:, None]
        u = u / vc.norm(u[:, :3])[:, None]
    return Transform(np.stack((w, v, u, pos), axis=2))


def from_perspective(*, pos=None, w=None, v=None, u=None, vol=None, ignore_scale=True):
    """Transform from world coordinates to the frame ``(pos; w, v, u)``."""
    return to_perspective(pos=pos, w=w, v=v, u=u, vol=vol, ignore_scale=ignore_scale).inv


def random_transform():
    """A random rotation * scaling * translation (test helper)."""
    t, pos, axis, s = np.random.normal(size=(4, 3))
    angle = np.random.normal()
    return rotate(pos=pos, axis=axis, angles=angle) * scale(abs(s)) * translate(t)
