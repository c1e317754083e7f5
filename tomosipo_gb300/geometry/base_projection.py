"""Common base of projection geometries (``tomosipo/geometry/base_projection.py``).

Projection geometries are indexed ``(angle, v, u)``; their data is stored as a
sinogram stack ``(v, angle, u)`` (``doc/topics/geometries.rst:39-49``).
"""
from .. import types


def is_projection(g):
    return isinstance(g, ProjectionGeometry)


def is_cone(g):
    return is_projection(g) and g.is_cone


def is_parallel(g):
    return is_projection(g) and g.is_parallel


class ProjectionGeometry:
    _is_cone = False
    _is_parallel = False
    _is_vector = False

    def __init__(self, shape=1):
        self._shape = types.to_shape2d(shape)

    def __len__(self):
        return self.num_steps

    @property
    def is_cone(self):
        return self._is_cone

    @property
    def is_parallel(self):
        return self._is_parallel

    @property
    def is_vec(self):
        return self._is_vector

    @property
    def det_shape(self):
        """(height, width) of the detector in pixels."""
        return self._shape

    @property
    def num_steps(self):
        return self.num_angles

    @property
    def num_angles(self):
        raise NotImplementedError()

    @property
    def angles(self):
        raise NotImplementedError()

    @property
    def src_pos(self):
        raise NotImplementedError()

    @property
    def ray_dir(self):
        raise NotImplementedError()

    def to_vec(self):
        raise NotImplementedError()

    def to_astra(self):
        raise NotImplementedError()

    # The properties below are answered by the vector form.
    @property
    def det_pos(self):
        return self.to_vec().det_pos

    @property
    def det_v(self):
        return self.to_vec().det_v

    @property
    def det_u(self):
        return self.to_vec().det_u

    @property
    def det_normal(self):
        return self.to_vec().det_normal

    @property
    def det_size(self):
        return self.to_vec().det_size

    @property
    def det_sizes(self):
        return self.to_vec().det_sizes

    @property
    def corners(self):
        return self.to_vec().corners

    @property
    def lower_left_corner(self):
        return self.to_vec().lower_left_corner

    def project_point(self, point):
        return self.to_vec().project_point(point)

    def to_vol(self):
        return self.to_vec().to_vol()
