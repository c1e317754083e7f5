"""Arbitrarily oriented (vector) volume geometry.

API of tomosipo's ``tomosipo/geometry/volume_vec.py``: a box of
``shape`` voxels centred on ``pos`` whose voxel axes are the vectors
``w, v, u`` (one row per time step). Voxel ``(i, j, k)`` is centred at
``lower_left_corner + (i + 1/2) w + (j + 1/2) v + (k + 1/2) u``
(``volume_vec.py:353-399``).
"""
from numbers import Integral

import numpy as np

from .. import types
from .. import vector_calc as vc
from ..utils import slice_interval, print_options
from .transform import Transform, EPSILON


def volume_vec(*, shape, pos=0, w=(1, 0, 0), v=(0, 1, 0), u=(0, 0, 1)):
    """Create an arbitrarily oriented volume geometry."""
    return VolumeVectorGeometry(shape, pos, w, v, u)


def random_volume_vec():
    from .transform import random_transform

    vg = volume_vec(
        shape=np.random.uniform(4, 10, size=3).astype(int),
        pos=np.random.normal(size=3),
    )
    return random_transform() * vg


class VolumeVectorGeometry:
    def __init__(self, shape, pos, w=(1, 0, 0), v=(0, 1, 0), u=(0, 0, 1)):
        self._shape = types.to_shape3d(shape)
        if np.isscalar(pos) and pos == 0.0:
            pos = (0.0, 0.0, 0.0)
        pos = types.to_vec(pos, "position")
        w = types.to_vec(w, "w axis")
        v = types.to_vec(v, "v axis")
        u = types.to_vec(u, "u axis")
        shapes = {x.shape[0] for x in (pos, w, v, u)} - {1}
        if len(shapes) > 1:
            raise ValueError(
                "Not all arguments pos, w, v, u are the same shape. "
                f"Got: {[x.shape for x in (pos, w, v, u)]}"
            )
        pos, w, v, u = (np.array(x) for x in np.broadcast_arrays(pos, w, v, u))
        self._pos, self._w, self._v, self._u = pos, w, v, u

    def __repr__(self):
        with print_options():
            return (
                "ts.volume_vec(\n"
                f"    shape={self._shape},\n"
                f"    pos={self._pos!r},\n"
                f"    w={self._w!r},\n"
                f"    v={self._v!r},\n"
                f"    u={self._u!r},\n"
                ")"
            )

    def __eq__(self, other):
        if not isinstance(other, VolumeVectorGeometry):
            return False
        if self.shape != other.shape or len(self) != len(other):
            return False
        return all(
            np.all(np.abs(a - b) < EPSILON)
            for a, b in [
                (self._pos, other._pos),
                (self._w, other._w),
                (self._v, other._v),
                (self._u, other._u),
            ]
        )

    def __len__(self):
        return self.num_steps

    def __getitem__(self, key):
        """Index ``[step, w, v, u]``; spatial slices bin voxels (see slice_interval)."""
        full = slice(None)
        if isinstance(key, (Integral, np.integer, slice)):
            key = (key, full, full, full)
        if isinstance(key, tuple):
            if len(key) > 4:
                raise ValueError(
                    f"VolumeVectorGeometry supports indexing in 4 dimensions. Got {key}."
                )
            key = key + (full,) * (4 - len(key))
            lims = [
                slice_interval(0, n, n, k) for n, k in zip(self._shape, key[1:])
            ]
            (w0, w1, lw, sw), (v0, v1, lv, sv), (u0, u1, lu, su) = lims
            llc = self.lower_left_corner
            new_llc = llc + w0 * self._w + v0 * self._v + u0 * self._u
            new_trc = llc + w1 * self._w + v1 * self._v + u1 * self._u
            step = key[0]
            if isinstance(step, (Integral, np.integer)):
                step = slice(int(step), int(step) + 1 if int(step) != -1 else None)
            new_pos = ((new_llc + new_trc) / 2)[step]
            return VolumeVectorGeometry(
                (lw, lv, lu),
                new_pos,
                sw * self._w[step],
                sv * self._v[step],
                su * self._u[step],
            )
        # boolean / integer array over steps
        return VolumeVectorGeometry(
            self._shape, self._pos[key], self._w[key], self._v[key], self._u[key]
        )

    def to_vec(self):
        return self

    # Properties ------------------------------------------------------------
    @property
    def num_steps(self):
        return len(self._pos)

    @property
    def pos(self):
        return self._pos.copy()

    @property
    def w(self):
        return self._w.copy()

    @property
    def v(self):
        return self._v.copy()

    @property
    def u(self):
        return self._u.copy()

    @property
    def shape(self):
        return self._shape

    @property
    def sizes(self):
        """(num_steps, 3) absolute sizes along w, v, u."""
        return np.stack(
            [n * vc.norm(x) for n, x in zip(self._shape, (self._w, self._v, self._u))],
            axis=1,
        )

    @property
    def size(self):
        s = self.sizes
        if np.all(np.ptp(s, axis=0) < EPSILON):
            return tuple(float(x) for x in s[0])
        raise ValueError(
            "The size of the volume is not constant. "
            "To prevent this error, use `vg.sizes'. "
        )

    @property
    def voxel_sizes(self):
        return self.sizes / np.array([self._shape])

    @property
    def voxel_size(self):
        return tuple(sz / n for sz, n in zip(self.size, self._shape))

    @property
    def corners(self):
        """(num_steps, 8, 3) corners, in the order (w, v, u) in {0,1}^3."""
        c = np.array([(a, b, d) for a in (0, 1) for b in (0, 1) for d in (0, 1)]) - 0.5
        n = self._shape
        pts = (
            self._pos[:, None, :]
            + c[None, :, 0:1] * self._w[:, None, :] * n[0]
            + c[None, :, 1:2] * self._v[:, None, :] * n[1]
            + c[None, :, 2:3] * self._u[:, None, :] * n[2]
        )
        return pts

    @property
    def lower_left_corner(self):
        n = self._shape
        return self._pos - (self._w * n[0] + self._v * n[1] + self._u * n[2]) / 2

    # Transformations -------------------------------------------------------
    def reshape(self, new_shape):
        """Change the number of voxels, keeping the physical box."""
        new_shape = types.to_shape3d(new_shape)
        sizes = self.sizes
        axes = [self._w, self._v, self._u]
        new_axes = [
            axes[i] / vc.norm(axes[i])[:, None] * (sizes[:, i] / max(new_shape[i], 1))[:, None]
            for i in range(3)
        ]
        return VolumeVectorGeometry(new_shape, self._pos, *new_axes)

    def __rmul__(self, other):
        if isinstance(other, Transform):
            return VolumeVectorGeometry(
                self._shape,
                other.transform_point(self._pos),
                other.transform_vec(self._w),
                other.transform_vec(self._v),
                other.transform_vec(self._u),
            )
        return NotImplemented
