"""Arbitrarily oriented cone-beam geometry: ``ts.cone_vec``.

API of tomosipo's ``tomosipo/geometry/cone_vec.py:10-339``. Per angle: source
position ``src_pos``, detector centre ``det_pos`` and pixel vectors ``det_v``,
``det_u`` in ``(z, y, x)``. ASTRA's ``cone_vec`` row is
``[src, det_pos, det_u, det_v]`` in ``(x, y, z)`` (``cone_vec.py:174-191``).
"""
import numpy as np

from .. import types
from .base_projection import ProjectionGeometry
from .det_vec import DetectorVectorGeometry
from .transform import Transform, EPSILON


def cone_vec(*, shape, src_pos, det_pos, det_v, det_u):
    return ConeVectorGeometry(
        shape=shape, src_pos=src_pos, det_pos=det_pos, det_v=det_v, det_u=det_u
    )


def random_cone_vec():
    from .cone import random_cone
    from .transform import random_transform

    return random_transform() * random_cone().to_vec()


class ConeVectorGeometry(ProjectionGeometry):
    _is_cone = True
    _is_vector = True

    def __init__(self, *, shape, src_pos, det_pos, det_v, det_u):
        super().__init__(shape=shape)
        src_pos = types.to_vec(src_pos, "source position")
        det_pos = types.to_vec(det_pos, "detector position")
        det_v = types.to_vec(det_v, "v axis")
        det_u = types.to_vec(det_u, "u axis")
        lens = {len(x) for x in (src_pos, det_pos, det_v, det_u)} - {1}
        if len(lens) > 1:
            raise ValueError(
                "Not all arguments src_pos, det_pos, det_v, det_u are the same shape. "
                f"Got: {[x.shape for x in (src_pos, det_pos, det_v, det_u)]}"
            )
        src_pos, det_pos, det_v, det_u = (
            np.array(x) for x in np.broadcast_arrays(src_pos, det_pos, det_v, det_u)
        )
        self._src_pos = src_pos
        self._det_vec = DetectorVectorGeometry(shape, det_pos, det_v, det_u)

    def __repr__(self):
        from ..utils import print_options

        with print_options():
            return (
                "ts.cone_vec(\n"
                f"    shape={self.det_shape},\n"
                f"    src_pos={self._src_pos!r},\n"
                f"    det_pos={self._det_vec._det_pos!r},\n"
                f"    det_v={self._det_vec._det_v!r},\n"
                f"    det_u={self._det_vec._det_u!r},\n"
                ")"
            )

    def __eq__(self, other):
        if not isinstance(other, ConeVectorGeometry):
            return False
        return (
            self._det_vec == other._det_vec
            and bool(np.all(np.abs(self._src_pos - other._src_pos) < EPSILON))
        )

    def __getitem__(self, key):
        d = self._det_vec[key]
        return cone_vec(
            shape=d.det_shape,
            src_pos=self._src_pos[DetectorVectorGeometry._angle_key(key)],
            det_pos=d._det_pos,
            det_v=d._det_v,
            det_u=d._det_u,
        )

    def to_vec(self):
        return self

    def to_astra(self):
        rows, cols = self.det_shape
        return {
            "type": "cone_vec",
            "DetectorRowCount": rows,
            "DetectorColCount": cols,
            "Vectors": self._det_vec._astra_vectors(self._src_pos),
        }

    @staticmethod
    def from_astra(astra_pg):
        if astra_pg["type"] != "cone_vec":
            raise ValueError(
                "ConeVectorGeometry.from_astra only supports 'cone_vec' type astra geometries."
            )
        vec = np.asarray(astra_pg["Vectors"], dtype=np.float64)
        return cone_vec(
            shape=(astra_pg["DetectorRowCount"], astra_pg["DetectorColCount"]),
            src_pos=vec[:, 0:3][:, ::-1],
            det_pos=vec[:, 3:6][:, ::-1],
            det_u=vec[:, 6:9][:, ::-1],
            det_v=vec[:, 9:12][:, ::-1],
        )

    @property
    def num_angles(self):
        return self._det_vec.num_angles

    @property
    def src_pos(self):
        return self._src_pos.copy()

    @property
    def det_pos(self):
        return self._det_vec.det_pos

    @property
    def det_v(self):
        return self._det_vec.det_v

    @property
    def det_u(self):
        return self._det_vec.det_u

    @property
    def det_normal(self):
        return self._det_vec.det_normal

    @property
    def det_size(self):
        return self._det_vec.det_size

    @property
    def det_sizes(self):
        return self._det_vec.det_sizes

    @property
    def corners(self):
        return self._det_vec.corners

    @property
    def lower_left_corner(self):
        return self._det_vec.lower_left_corner

    def to_vol(self):
        return self._det_vec.to_vol()

    def rescale_det(self, scale):
        d = self._det_vec.rescale_det(scale)
        return cone_vec(
            shape=d.det_shape, src_pos=self._src_pos, det_pos=d._det_pos, det_v=d._det_v, det_u=d._det_u
        )

    def reshape(self, new_shape):
        d = self._det_vec.reshape(new_shape)
        return cone_vec(
            shape=d.det_shape, src_pos=self._src_pos, det_pos=d._det_pos, det_v=d._det_v, det_u=d._det_u
        )

    def project_point(self, point):
        """(v, u) detector coordinates, relative to the centre, of each point."""
        if np.isscalar(point):
            point = types.to_pos(point)
        p = types.to_vec(point)
        return self._det_vec._project(p, p - self._src_pos)

    def __rmul__(self, other):
        if isinstance(other, Transform):
            d = other * self._det_vec
            return cone_vec(
                shape=self.det_shape,
                src_pos=other.transform_point(self._src_pos),
                det_pos=d._det_pos,
                det_v=d._det_v,
                det_u=d._det_u,
            )
        return NotImplemented
