"""Circular parallel-beam geometry: ``ts.parallel``.

API of tomosipo's ``tomosipo/geometry/parallel.py:13-282``. An integer
``angles`` means ``linspace(0, pi, angles, endpoint=False)``
(``parallel.py:86-88``). ``to_vec`` uses ASTRA's public parallel3d -> vec
convention, which tomosipo's docs pin numerically
(``doc/topics/geometries.rst:364-410``): in ``(z, y, x)``,
``ray = (0, -cos t, sin t)``, ``det_pos = 0``, ``det_u = (0, sin t, cos t) * su``,
``det_v = (sv, 0, 0)``.
"""
import warnings

import numpy as np

from .. import types
from .base_projection import ProjectionGeometry
from .parallel_vec import parallel_vec
from .transform import Transform, EPSILON


def parallel(*, angles=1, shape=1, size=None):
    return ParallelGeometry(angles, shape, size)


def random_parallel():
    return parallel(
        angles=np.random.normal(size=20),
        shape=np.random.uniform(10, 20, size=2).astype(int),
        size=np.random.uniform(10, 20, size=2),
    )


class ParallelGeometry(ProjectionGeometry):
    _is_parallel = True

    def __init__(self, angles=1, shape=1, size=None):
        super().__init__(shape=shape)
        self._angles_original = angles
        if np.isscalar(angles) and isinstance(angles, (int, np.integer)) and not isinstance(angles, bool):
            angles = np.linspace(0, np.pi, int(angles), endpoint=False)
        else:
            angles = types.to_scalars(angles, var_name="angles", accept_empty=True)
        if len(angles) == 0:
            raise TypeError(
                f"ParallelGeometry expects non-empty array of angles; got {self._angles_original}"
            )
        self._angles = angles
        self._size = types.to_size2d(self.det_shape if size is None else size)

    def __repr__(self):
        from ..utils import print_options

        with print_options():
            return (
                "ts.parallel(\n"
                f"    angles={self._angles_original!r},\n"
                f"    shape={self.det_shape!r},\n"
                f"    size={self._size!r},\n"
                ")"
            )

    def __eq__(self, other):
        if not isinstance(other, ParallelGeometry):
            return False
        return (
            self.det_shape == other.det_shape
            and len(self._angles) == len(other._angles)
            and bool(np.all(np.abs(self._angles - other._angles) < EPSILON))
            and bool(np.all(np.abs(np.array(self._size) - other._size) < EPSILON))
        )

    def __getitem__(self, key):
        if isinstance(key, tuple):
            raise ValueError(
                f"Expected 1 index to ParallelGeometry, got {len(key)}. "
                "Indexing on the detector plane is not supported, "
                "since it might move the detector center. "
                "To prevent this error, use `pg.to_vec()[a:b, c:d, e:f]'. "
            )
        return parallel(
            angles=np.array(self._angles[key], ndmin=1), shape=self.det_shape, size=self._size
        )

    def to_vec(self):
        t = self._angles
        sv = self._size[0] / self.det_shape[0]
        su = self._size[1] / self.det_shape[1]
        zero = np.zeros_like(t)
        c, s = np.cos(t), np.sin(t)
        return parallel_vec(
            shape=self.det_shape,
            ray_dir=np.stack([zero, -c, s], axis=1),
            det_pos=np.zeros((len(t), 3)),
            det_v=np.stack([zero + sv, zero, zero], axis=1),
            det_u=np.stack([zero, s * su, c * su], axis=1),
        )

    def to_astra(self):
        rows, cols = self.det_shape
        return {
            "type": "parallel3d",
            "DetectorSpacingX": self._size[1] / cols,
            "DetectorSpacingY": self._size[0] / rows,
            "DetectorRowCount": rows,
            "DetectorColCount": cols,
            "ProjectionAngles": self._angles.copy(),
        }

    @staticmethod
    def from_astra(astra_pg):
        if astra_pg["type"] != "parallel3d":
            raise ValueError(
                "ParallelGeometry.from_astra only supports 'parallel3d' type astra geometries."
            )
        shape = (astra_pg["DetectorRowCount"], astra_pg["DetectorColCount"])
        spacing = (astra_pg["DetectorSpacingY"], astra_pg["DetectorSpacingX"])
        return parallel(
            angles=np.array(astra_pg["ProjectionAngles"], dtype=np.float64),
            shape=shape,
            size=tuple(np.array(spacing) * np.array(shape)),
        )

    @property
    def num_angles(self):
        return len(self._angles)

    @property
    def angles(self):
        return self._angles.copy()

    @property
    def ray_dir(self):
        return self.to_vec().ray_dir

    @property
    def det_size(self):
        return self._size

    @property
    def det_sizes(self):
        return np.repeat([self._size], self.num_angles, axis=0)

    def rescale_det(self, scale):
        sv, su = (int(x) for x in types.to_size2d(scale))
        shape = (self.det_shape[0] // sv, self.det_shape[1] // su)
        return parallel(angles=self._angles.copy(), shape=shape, size=self._size)

    def reshape(self, new_shape):
        return parallel(angles=self._angles.copy(), shape=new_shape, size=self._size)

    def __rmul__(self, other):
        if isinstance(other, Transform):
            warnings.warn(
                "Converting parallel geometry to vector geometry. "
                "Use `T * pg.to_vec()` to inhibit this warning. ",
                stacklevel=2,
            )
            return other * self.to_vec()
        return NotImplemented
