"""Axis-aligned volume geometry: ``ts.volume``.

API of tomosipo's ``tomosipo/geometry/volume.py:35-127``: a box of ``shape``
voxels ``(z, y, x)``, centred on ``pos``, of physical ``size`` (default: equal
to ``shape``), or given by ``extent``. Voxel ``i`` along an axis is centred at
``pos - size/2 + (i + 1/2) * size/shape``.
"""
import warnings

import numpy as np

from .. import types
from .transform import Transform, translate, scale as _scale
from .volume_vec import VolumeVectorGeometry


def is_volume(g):
    return isinstance(g, (VolumeGeometry, VolumeVectorGeometry))


def _pos_size_to_extent(pos, size):
    pos = np.array(types.to_pos(pos))
    size = np.array(types.to_size3d(size))
    return tuple((float(p - s / 2), float(p + s / 2)) for p, s in zip(pos, size))


def _extent_to_pos_size(extent):
    # three (low, high) pairs, one per axis; anything else is a TypeError, as in
    # tomosipo/geometry/volume.py:154-158
    try:
        extent = np.array(extent, dtype=np.float64)
    except (TypeError, ValueError):
        raise TypeError(f"Expected an extent of three (low, high) pairs. Got {extent!r}.")
    if extent.shape != (3, 2):
        raise TypeError(f"Expected an extent of three (low, high) pairs. Got shape {extent.shape}.")
    size = types.to_size3d(tuple(extent[:, 1] - extent[:, 0]))
    pos = types.to_pos(tuple((extent[:, 1] + extent[:, 0]) / 2))
    return pos, size


def volume(*, shape=(1, 1, 1), pos=None, size=None, extent=None):
    """Create an axis-aligned volume geometry."""
    shape = types.to_shape3d(shape)
    if extent is not None and pos is not None:
        raise ValueError("ts.volume does not accept both `extent` and `pos` arguments. ")
    if extent is not None and size is not None:
        raise ValueError("ts.volume does not accept both `extent` and `size` arguments. ")
    if extent is not None:
        pos, size = _extent_to_pos_size(extent)
    return VolumeGeometry(
        shape, pos=0 if pos is None else pos, size=shape if size is None else size
    )


def random_volume():
    return volume(
        shape=np.random.uniform(2, 100, 3).astype(int),
        pos=np.random.normal(size=3),
        size=np.random.uniform(1, 10, size=3),
    )


class VolumeGeometry:
    """A single-step, axis-aligned volume."""

    def __init__(self, shape=(1, 1, 1), pos=0, size=None):
        shape = types.to_shape3d(shape)
        pos = types.to_pos(pos)
        size = shape if size is None else types.to_size3d(size)
        vs = tuple(float(sz) / n if n > 0 else 0.0 for sz, n in zip(size, shape))
        self._inner = VolumeVectorGeometry(
            shape, pos, w=(vs[0], 0, 0), v=(0, vs[1], 0), u=(0, 0, vs[2])
        )

    def __repr__(self):
        return (
            "ts.volume(\n"
            f"    shape={self.shape},\n"
            f"    pos={tuple(float(x) for x in self.pos[0])},\n"
            f"    size={self.size},\n"
            ")"
        )

    def __eq__(self, other):
        return isinstance(other, VolumeGeometry) and self._inner == other._inner

    def __getitem__(self, key):
        inner = self._inner[(0, *key)] if isinstance(key, tuple) else self._inner[0, key]
        return VolumeGeometry(inner.shape, tuple(inner.pos[0]), inner.size)

    def __contains__(self, other):
        return all(
            s[0] <= o[0] and o[1] <= s[1] for s, o in zip(self.extent, other.extent)
        )

    def __len__(self):
        return 1

    def to_vec(self):
        return self._inner

    def to_astra(self):
        """ASTRA 3D volume geometry dict (``create_vol_geom`` layout)."""
        (z0, z1), (y0, y1), (x0, x1) = self.extent
        nz, ny, nx = self.shape
        return {
            "GridRowCount": ny,
            "GridColCount": nx,
            "GridSliceCount": nz,
            "option": {
                "WindowMinX": x0,
                "WindowMaxX": x1,
                "WindowMinY": y0,
                "WindowMaxY": y1,
                "WindowMinZ": z0,
                "WindowMaxZ": z1,
            },
        }

    # Properties ------------------------------------------------------------
    @property
    def num_steps(self):
        return 1

    @property
    def pos(self):
        return self._inner.pos

    @property
    def w(self):
        return self._inner.w

    @property
    def v(self):
        return self._inner.v

    @property
    def u(self):
        return self._inner.u

    @property
    def shape(self):
        return self._inner.shape

    @property
    def sizes(self):
        return self._inner.sizes

    @property
    def size(self):
        return self._inner.size

    @property
    def voxel_sizes(self):
        return self._inner.voxel_sizes

    @property
    def voxel_size(self):
        return self._inner.voxel_size

    @property
    def extent(self):
        return _pos_size_to_extent(tuple(self.pos[0]), self.size)

    @property
    def corners(self):
        return self._inner.corners

    @property
    def lower_left_corner(self):
        return self._inner.lower_left_corner

    # Transformations -------------------------------------------------------
    def with_voxel_size(self, voxel_size):
        voxel_size = np.array(types.to_size3d(voxel_size))
        new_shape = (np.array(self.size) / voxel_size).astype(int)
        return VolumeGeometry(tuple(new_shape), tuple(self.pos[0]), tuple(new_shape * voxel_size))

    def reshape(self, new_shape):
        return VolumeGeometry(new_shape, tuple(self.pos[0]), self.size)

    def translate(self, t):
        t = types.to_pos(t)
        return VolumeGeometry(
            self.shape, tuple(p + d for p, d in zip(self.pos[0], t)), self.size
        )

    def untranslate(self, t):
        return self.translate(tuple(-np.array(t, dtype=np.float64)))

    def scale(self, s):
        s = types.to_size3d(s)
        return VolumeGeometry(
            self.shape, tuple(self.pos[0]), tuple(a * b for a, b in zip(s, self.size))
        )

    def multiply(self, s):
        s = types.to_size3d(s)
        return VolumeGeometry(
            self.shape,
            tuple(a * b for a, b in zip(s, self.pos[0])),
            tuple(a * b for a, b in zip(s, self.size)),
        )

    def __rmul__(self, other):
        if not isinstance(other, Transform):
            return NotImplemented
        if other.num_steps == 1:
            t = other.matrix[0, :3, 3]
            s = np.abs(np.diag(other.matrix[0])[:3])
            if translate(t) * _scale(s) == other:
                return self.multiply(tuple(s)).translate(tuple(t))
        warnings.warn(
            "Converting VolumeGeometry to VolumeVectorGeometry. "
            "Use `T * vg.to_vec()` to inhibit this warning. ",
            stacklevel=2,
        )
        return other * self.to_vec()


def from_astra(astra_vol_geom):
    """VolumeGeometry from an ASTRA 3D volume geometry dict."""
    o = astra_vol_geom["option"]
    shape = (
        astra_vol_geom["GridSliceCount"],
        astra_vol_geom["GridRowCount"],
        astra_vol_geom["GridColCount"],
    )
    extent = (
        (o["WindowMinZ"], o["WindowMaxZ"]),
        (o["WindowMinY"], o["WindowMaxY"]),
        (o["WindowMinX"], o["WindowMaxX"]),
    )
    pos, size = _extent_to_pos_size(extent)
    return VolumeGeometry(shape, pos, size)
