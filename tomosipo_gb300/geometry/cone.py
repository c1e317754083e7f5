"""Circular cone-beam geometry: ``ts.cone``.

API of tomosipo's ``tomosipo/geometry/cone.py:13-399``. An integer ``angles``
means ``linspace(0, 2 pi, angles, endpoint=False)`` (``cone.py:164-166``).
``cone_angle`` sets ``src_orig_dist = src_det_dist = det_height / cone_angle``,
which places the detector through the origin (``cone.py:82-85``).

``to_vec`` uses ASTRA's public cone -> cone_vec convention: in ``(z, y, x)``,
``src = (0, -cos t, sin t) * d_so``, ``det_pos = (0, cos t, -sin t) * d_od``,
``det_u = (0, sin t, cos t) * su``, ``det_v = (sv, 0, 0)``, with
``d_od = src_det_dist - src_orig_dist`` (``cone.py:254-265``). The detector-plane
mapping and ``|src| = d_so`` are pinned by
``tests/geometry/test_cone_vec.py:143-201``.
"""
import warnings

import numpy as np

from .. import types
from .base_projection import ProjectionGeometry
from .cone_vec import cone_vec
from .transform import Transform, EPSILON


def cone(
    *,
    angles=1,
    shape=(1, 1),
    size=None,
    cone_angle=None,
    src_orig_dist=None,
    src_det_dist=None,
):
    shape = types.to_shape2d(shape)
    size = types.to_size2d(shape if size is None else size)
    if cone_angle is None and src_orig_dist is None and src_det_dist is None:
        raise ValueError(
            "ts.cone requires at least one of `cone_angle`, `src_orig_dist`, or `src_det_dist` parameters. "
        )
    if cone_angle is not None and src_orig_dist is not None:
        raise ValueError(
            "ts.cone does not accept both `cone_angle` and src_orig_dist` arguments at the same time. "
        )
    if cone_angle is not None and src_det_dist is not None:
        raise ValueError(
            "ts.cone does not accept both `cone_angle` and src_det_dist` arguments at the same time. "
        )
    if cone_angle is not None:
        src_det_dist = size[0] / cone_angle
        src_orig_dist = src_det_dist
    elif src_orig_dist is None:
        src_orig_dist = src_det_dist
    elif src_det_dist is None:
        src_det_dist = src_orig_dist
    return ConeGeometry(angles, shape, size, src_orig_dist, src_det_dist)


def random_cone():
    return cone(
        angles=np.random.normal(size=20),
        shape=np.random.uniform(10, 20, size=2).astype(int),
        size=np.random.uniform(10, 20, size=2),
        src_orig_dist=np.random.uniform(0, 10),
        src_det_dist=np.random.uniform(0, 20),
    )


class ConeGeometry(ProjectionGeometry):
    _is_cone = True

    def __init__(self, angles=1, shape=1, size=None, src_orig_dist=None, src_det_dist=None):
        super().__init__(shape=shape)
        self.angles_original = angles
        if np.isscalar(angles) and isinstance(angles, (int, np.integer)) and not isinstance(angles, bool):
            angles = np.linspace(0, 2 * np.pi, int(angles), endpoint=False)
        else:
            # an empty array is a TypeError here, an angle count of 0 a ValueError
            # below (tomosipo/geometry/cone.py:163-173)
            angles = types.to_scalars(angles, var_name="angles")
        if len(angles) == 0:
            raise ValueError(
                f"ConeGeometry expects non-empty array of angles; got {self.angles_original}"
            )
        if src_orig_dist is None:
            raise ValueError("Expected `src_orig_dist` parameter. Got `None`. ")
        if src_det_dist is None:
            raise ValueError("Expected `src_det_dist` parameter. Got `None`. ")
        self._angles = angles
        self._size = types.to_size2d(self.det_shape if size is None else size)
        self._src_orig_dist = float(src_orig_dist)
        self._src_det_dist = float(src_det_dist)

    def __repr__(self):
        from ..utils import print_options

        with print_options():
            return (
                "ts.cone(\n"
                f"    angles={self.angles_original!r},\n"
                f"    shape={self.det_shape},\n"
                f"    size={self.det_size},\n"
                f"    src_orig_dist={self._src_orig_dist},\n"
                f"    src_det_dist={self._src_det_dist},\n"
                ")"
            )

    def __eq__(self, other):
        if not isinstance(other, ConeGeometry):
            return False
        return (
            len(self._angles) == len(other._angles)
            and self.det_shape == other.det_shape
            and bool(np.all(np.abs(self._angles - other._angles) < EPSILON))
            and bool(np.all(np.abs(np.array(self._size) - other._size) < EPSILON))
            and abs(self._src_orig_dist - other._src_orig_dist) < EPSILON
            and abs(self._src_det_dist - other._src_det_dist) < EPSILON
        )

    def __getitem__(self, key):
        if isinstance(key, tuple):
            raise ValueError(
                f"Expected 1 index to ConeGeometry, got {len(key)}. "
                "Indexing on the detector plane is not supported, "
                "since it might move the detector center. "
            )
        return ConeGeometry(
            np.array(self._angles[key], ndmin=1),
            self.det_shape,
            self._size,
            self._src_orig_dist,
            self._src_det_dist,
        )

    def to_vec(self):
        t = self._angles
        sv = self._size[0] / self.det_shape[0]
        su = self._size[1] / self.det_shape[1]
        d_so = self._src_orig_dist
        d_od = self._src_det_dist - self._src_orig_dist
        zero = np.zeros_like(t)
        c, s = np.cos(t), np.sin(t)
        return cone_vec(
            shape=self.det_shape,
            src_pos=np.stack([zero, -c * d_so, s * d_so], axis=1),
            det_pos=np.stack([zero, c * d_od, -s * d_od], axis=1),
            det_v=np.stack([zero + sv, zero, zero], axis=1),
            det_u=np.stack([zero, s * su, c * su], axis=1),
        )

    def to_astra(self):
        rows, cols = self.det_shape
        return {
            "type": "cone",
            "DetectorSpacingX": self._size[1] / cols,
            "DetectorSpacingY": self._size[0] / rows,
            "DetectorRowCount": rows,
            "DetectorColCount": cols,
            "ProjectionAngles": self._angles.copy(),
            "DistanceOriginSource": self._src_orig_dist,
            "DistanceOriginDetector": self._src_det_dist - self._src_orig_dist,
        }

    @staticmethod
    def from_astra(astra_pg):
        if astra_pg["type"] != "cone":
            raise ValueError(
                "ConeGeometry.from_astra only supports 'cone' type astra geometries."
            )
        shape = (astra_pg["DetectorRowCount"], astra_pg["DetectorColCount"])
        spacing = (astra_pg["DetectorSpacingY"], astra_pg["DetectorSpacingX"])
        d_so = astra_pg["DistanceOriginSource"]
        return ConeGeometry(
            np.array(astra_pg["ProjectionAngles"], dtype=np.float64),
            shape,
            tuple(np.array(spacing) * np.array(shape)),
            d_so,
            d_so + astra_pg["DistanceOriginDetector"],
        )

    @property
    def src_orig_dist(self):
        return self._src_orig_dist

    @property
    def src_det_dist(self):
        return self._src_det_dist

    @property
    def num_angles(self):
        return len(self._angles)

    @property
    def angles(self):
        return self._angles.copy()

    @property
    def src_pos(self):
        return self.to_vec().src_pos

    @property
    def det_size(self):
        return self._size

    @property
    def det_sizes(self):
        return np.repeat([self._size], self.num_angles, axis=0)

    def rescale_det(self, scale):
        sv, su = (int(x) for x in types.to_size2d(scale))
        shape = (self.det_shape[0] // sv, self.det_shape[1] // su)
        return ConeGeometry(
            self.angles_original, shape, self._size, self._src_orig_dist, self._src_det_dist
        )

    def reshape(self, new_shape):
        return ConeGeometry(
            self.angles_original,
            types.to_shape2d(new_shape),
            self._size,
            self._src_orig_dist,
            self._src_det_dist,
        )

    def __rmul__(self, other):
        if isinstance(other, Transform):
            warnings.warn(
                "Converting cone geometry to vector geometry. "
                "Use `T * pg.to_vec()` to inhibit this warning. ",
                stacklevel=2,
            )
            return other * self.to_vec()
        return NotImplemented
