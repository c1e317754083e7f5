"""Detector-only vector geometry shared by ``parallel_vec`` and ``cone_vec``.

Same conventions as tomosipo's ``tomosipo/geometry/det_vec.py``: ``det_pos`` is
the detector centre, ``det_v`` / ``det_u`` step one pixel up / sideways, and
pixel ``(iv, iu)`` is centred at
``det_pos + (iv + 1/2 - rows/2) det_v + (iu + 1/2 - cols/2) det_u``.
"""
from numbers import Integral

import numpy as np

from .. import types
from .. import vector_calc as vc
from ..utils import slice_interval
from .base_projection import ProjectionGeometry
from .transform import Transform, EPSILON


def det_vec(shape, det_pos, det_v, det_u):
    return DetectorVectorGeometry(shape, det_pos, det_v, det_u)


def random_det_vec():
    shape = np.random.uniform(10, 20, size=2).astype(int)
    n = int(np.random.uniform(1, 100))
    return det_vec(shape, *np.random.normal(size=(3, n, 3)))


class DetectorVectorGeometry(ProjectionGeometry):
    _is_vector = True

    def __init__(self, shape, det_pos, det_v, det_u):
        super().__init__(shape=shape)
        det_pos, det_v, det_u = (types.to_vec(x) for x in (det_pos, det_v, det_u))
        lens = {len(x) for x in (det_pos, det_v, det_u)} - {1}
        if len(lens) > 1:
            raise ValueError(
                "Not all arguments det_pos, det_v, det_u are the same shape. "
                f"Got: {[x.shape for x in (det_pos, det_v, det_u)]}"
            )
        self._det_pos, self._det_v, self._det_u = (
            np.array(x) for x in np.broadcast_arrays(det_pos, det_v, det_u)
        )

    def __repr__(self):
        return (
            "DetectorVectorGeometry(\n"
            f"    shape={self.det_shape},\n"
            f"    det_pos={self._det_pos},\n"
            f"    det_v={self._det_v},\n"
            f"    det_u={self._det_u}\n"
            ")"
        )

    def __eq__(self, other):
        if not isinstance(other, DetectorVectorGeometry):
            return False
        if self.det_shape != other.det_shape or self.num_angles != other.num_angles:
            return False
        return all(
            np.all(np.abs(a - b) < EPSILON)
            for a, b in [
                (self._det_pos, other._det_pos),
                (self._det_v, other._det_v),
                (self._det_u, other._det_u),
            ]
        )

    def __getitem__(self, key):
        """Index ``[angle, v, u]``; detector slices bin pixels."""
        full = slice(None)
        if isinstance(key, (Integral, np.integer, slice)):
            key = (key, full, full)
        if isinstance(key, tuple):
            key = key + (full,) * (3 - len(key))
            if len(key) != 3:
                raise ValueError(f"Expected at most 3 indices. Got {key}.")
            v0, v1, lv, sv = slice_interval(0, self.det_shape[0], self.det_shape[0], key[1])
            u0, u1, lu, su = slice_interval(0, self.det_shape[1], self.det_shape[1], key[2])
            llc = self.lower_left_corner
            lo = llc + v0 * self._det_v + u0 * self._det_u
            hi = llc + v1 * self._det_v + u1 * self._det_u
            a = key[0]
            if isinstance(a, (Integral, np.integer)):
                a = slice(int(a), int(a) + 1 if int(a) != -1 else None)
            return det_vec((lv, lu), ((lo + hi) / 2)[a], self._det_v[a] * sv, self._det_u[a] * su)
        return det_vec(self.det_shape, self._det_pos[key], self._det_v[key], self._det_u[key])

    @staticmethod
    def _angle_key(key):
        if isinstance(key, tuple):
            key = key[0]
        if isinstance(key, (Integral, np.integer)):
            key = slice(int(key), int(key) + 1 if int(key) != -1 else None)
        return key

    def to_vec(self):
        return self

    def to_vol(self):
        """The detector as a one-voxel-thick volume vector geometry."""
        from .volume_vec import volume_vec

        n = self.det_normal
        return volume_vec(
            shape=(self.det_shape[0], 1, self.det_shape[1]),
            pos=self._det_pos,
            w=self._det_v,
            v=n / vc.norm(n)[:, None],
            u=self._det_u,
        )

    def to_astra(self):
        """ASTRA-style dict of the detector alone (tomosipo's ``det_vec`` pseudo-type,
        ``tomosipo/geometry/det_vec.py:180-199``): the vector rows of a
        ``*_vec`` geometry with zeros where the source or ray direction goes."""
        rows, cols = self.det_shape
        return {
            "type": "det_vec",
            "DetectorRowCount": rows,
            "DetectorColCount": cols,
            "Vectors": self._astra_vectors(np.zeros_like(self._det_pos)),
        }

    @staticmethod
    def from_astra(astra_pg):
        if astra_pg["type"] != "det_vec":
            raise ValueError(
                "DetectorVectorGeometry.from_astra only supports 'det_vec' type astra geometries."
            )
        vec = np.asarray(astra_pg["Vectors"], dtype=np.float64)
        return det_vec(
            (astra_pg["DetectorRowCount"], astra_pg["DetectorColCount"]),
            det_pos=vec[:, 3:6][:, ::-1],
            det_v=vec[:, 9:12][:, ::-1],
            det_u=vec[:, 6:9][:, ::-1],
        )

    def _astra_vectors(self, first):
        return np.concatenate(
            [first[:, ::-1], self._det_pos[:, ::-1], self._det_u[:, ::-1], self._det_v[:, ::-1]],
            axis=1,
        )

    # Properties ------------------------------------------------------------
    @property
    def num_angles(self):
        return len(self._det_pos)

    @property
    def det_pos(self):
        return self._det_pos.copy()

    @property
    def det_v(self):
        return self._det_v.copy()

    @property
    def det_u(self):
        return self._det_u.copy()

    @property
    def det_normal(self):
        return vc.cross_product(self._det_u, self._det_v)

    @property
    def det_sizes(self):
        h = vc.norm(self._det_v) * self.det_shape[0]
        w = vc.norm(self._det_u) * self.det_shape[1]
        return np.stack([h, w], axis=1)

    @property
    def det_size(self):
        s = self.det_sizes
        if np.all(np.ptp(s, axis=0) < EPSILON):
            return (float(s[0, 0]), float(s[0, 1]))
        raise ValueError(
            "The size of the detector is not constant. "
            "To prevent this error, use `pg.det_sizes'. "
        )

    @property
    def corners(self):
        """(num_angles, 4, 3): (-u,-v), (-u,+v), (+u,-v), (+u,+v) corners."""
        du = self._det_u * self.det_shape[1] / 2
        dv = self._det_v * self.det_shape[0] / 2
        p = self._det_pos
        return np.stack([p - du - dv, p - du + dv, p + du - dv, p + du + dv], axis=1)

    @property
    def lower_left_corner(self):
        return (
            self._det_pos
            - self._det_v * self.det_shape[0] / 2
            - self._det_u * self.det_shape[1] / 2
        )

    # Transformations -------------------------------------------------------
    def rescale_det(self, scale):
        sv, su = (int(x) for x in types.to_size2d(scale))
        shape = (self.det_shape[0] // sv, self.det_shape[1] // su)
        return det_vec(shape, self._det_pos, self._det_v * sv, self._det_u * su)

    def reshape(self, new_shape):
        new_shape = types.to_shape2d(new_shape)
        return det_vec(
            new_shape,
            self._det_pos,
            self._det_v * self.det_shape[0] / new_shape[0],
            self._det_u * self.det_shape[1] / new_shape[1],
        )

    def project_point(self, point):
        """A detector alone has no source or ray direction to project along
        (tomosipo raises the same)."""
        raise NotImplementedError()

    def _project(self, origin, direction):
        point = types.to_vec(origin)
        hit = vc.intersect(point, direction, self._det_pos, self.det_normal)
        rel = hit - self._det_pos
        iu = vc.dot(rel, self._det_u) / vc.squared_norm(self._det_u)
        iv = vc.dot(rel, self._det_v) / vc.squared_norm(self._det_v)
        return np.stack((iv, iu), axis=-1)

    def __rmul__(self, other):
        if isinstance(other, Transform):
            return det_vec(
                self.det_shape,
                other.transform_point(self._det_pos),
                other.transform_vec(self._det_v),
                other.transform_vec(self._det_u),
            )
        return NotImplemented
