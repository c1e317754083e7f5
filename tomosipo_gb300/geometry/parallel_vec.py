"""Arbitrarily oriented parallel-beam geometry: ``ts.parallel_vec``.

API of tomosipo's ``tomosipo/geometry/parallel_vec.py:15-343``. Per angle:
``ray_dir``, detector centre ``det_pos`` and pixel vectors ``det_v``, ``det_u``,
all in ``(z, y, x)``. ASTRA's ``parallel3d_vec`` row is
``[ray, det_pos, det_u, det_v]`` with each vector in ``(x, y, z)``
(``parallel_vec.py:175-192``).
"""
import numpy as np

from .. import types
from .base_projection import ProjectionGeometry
from .det_vec import DetectorVectorGeometry
from .transform import Transform, EPSILON


def parallel_vec(*, shape, ray_dir, det_pos, det_v, det_u):
    return ParallelVectorGeometry(shape, ray_dir, det_pos, det_v, det_u)


def random_parallel_vec():
    n = int(np.random.uniform(1, 20))
    return parallel_vec(
        shape=np.random.uniform(10, 20, size=2).astype(int),
        ray_dir=np.random.normal(size=(n, 3)),
        det_pos=np.random.normal(size=(n, 3)),
        det_v=np.random.normal(size=(n, 3)),
        det_u=np.random.normal(size=(n, 3)),
    )


class ParallelVectorGeometry(ProjectionGeometry):
    _is_parallel = True
    _is_vector = True

    def __init__(self, shape, ray_dir, det_pos, det_v, det_u):
        super().__init__(shape=shape)
        ray_dir = types.to_vec(ray_dir, "ray direction")
        det_pos = types.to_vec(det_pos, "detector position")
        det_v = types.to_vec(det_v, "v axis")
        det_u = types.to_vec(det_u, "u axis")
        lens = {len(x) for x in (ray_dir, det_pos, det_v, det_u)} - {1}
        if len(lens) > 1:
            raise ValueError(
                "Not all arguments ray_dir, det_pos, det_v, det_u are the same shape. "
                f"Got: {[x.shape for x in (ray_dir, det_pos, det_v, det_u)]}"
            )
        ray_dir, det_pos, det_v, det_u = (
            np.array(x) for x in np.broadcast_arrays(ray_dir, det_pos, det_v, det_u)
        )
        self._ray_dir = ray_dir
        self._det_vec = DetectorVectorGeometry(shape, det_pos, det_v, det_u)

    def __repr__(self):
        from ..utils import print_options

        with print_options():
            return (
                "ts.parallel_vec(\n"
                f"    shape={self.det_shape},\n"
                f"    ray_dir={self._ray_dir!r},\n"
                f"    det_pos={self._det_vec._det_pos!r},\n"
                f"    det_v={self._det_vec._det_v!r},\n"
                f"    det_u={self._det_vec._det_u!r},\n"
                ")"
            )

    def __eq__(self, other):
        if not isinstance(other, ParallelVectorGeometry):
            return False
        return (
            self._det_vec == other._det_vec
            and self._ray_dir.shape == other._ray_dir.shape
            and bool(np.all(np.abs(self._ray_dir - other._ray_dir) < EPSILON))
        )

    def __getitem__(self, key):
        d = self._det_vec[key]
        return parallel_vec(
            shape=d.det_shape,
            ray_dir=self._ray_dir[DetectorVectorGeometry._angle_key(key)],
            det_pos=d._det_pos,
            det_v=d._det_v,
            det_u=d._det_u,
        )

    def to_vec(self):
        return self

    def to_astra(self):
        rows, cols = self.det_shape
        return {
            "type": "parallel3d_vec",
            "DetectorRowCount": rows,
            "DetectorColCount": cols,
            "Vectors": self._det_vec._astra_vectors(self._ray_dir),
        }

    @staticmethod
    def from_astra(astra_pg):
        if astra_pg["type"] != "parallel3d_vec":
            raise ValueError(
                "ParallelVectorGeometry.from_astra only supports 'parallel3d_vec' type astra geometries."
            )
        vec = np.asarray(astra_pg["Vectors"], dtype=np.float64)
        return parallel_vec(
            shape=(astra_pg["DetectorRowCount"], astra_pg["DetectorColCount"]),
            ray_dir=vec[:, 0:3][:, ::-1],
            det_pos=vec[:, 3:6][:, ::-1],
            det_u=vec[:, 6:9][:, ::-1],
            det_v=vec[:, 9:12][:, ::-1],
        )

    @property
    def num_angles(self):
        return self._det_vec.num_angles

    @property
    def ray_dir(self):
        return self._ray_dir.copy()

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
        return parallel_vec(
            shape=d.det_shape, ray_dir=self._ray_dir, det_pos=d._det_pos, det_v=d._det_v, det_u=d._det_u
        )

    def reshape(self, new_shape):
        d = self._det_vec.reshape(new_shape)
        return parallel_vec(
            shape=d.det_shape, ray_dir=self._ray_dir, det_pos=d._det_pos, det_v=d._det_v, det_u=d._det_u
        )

    def project_point(self, point):
        """(v, u) detector coordinates, relative to the centre, of each point."""
        if np.isscalar(point):
            point = types.to_pos(point)
        return self._det_vec._project(point, self._ray_dir)

    def __rmul__(self, other):
        if isinstance(other, Transform):
            d = other * self._det_vec
            return parallel_vec(
                shape=self.det_shape,
                ray_dir=other.transform_vec(self._ray_dir),
                det_pos=d._det_pos,
                det_v=d._det_v,
                det_u=d._det_u,
            )
        return NotImplemented
