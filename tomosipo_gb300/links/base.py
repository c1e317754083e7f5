"""Array links: wrap user arrays for projection (``tomosipo/links/base.py``).

``link(geometry, arr)`` picks the first backend that accepts ``arr``;
``geometry_shape`` gives the array shape a geometry expects: a volume's
``shape``, or ``(det_rows, num_angles, det_cols)`` for a projection geometry
(``tomosipo/links/base.py:21-31``).
"""
import warnings
from contextlib import contextmanager

backends = []


def link(geometry, arr):
    shape = geometry_shape(geometry)
    for backend in backends:
        if backend.__accepts__(arr):
            return backend(shape, arr)
    raise ValueError(f"An initial_value of class {type(arr)} is not supported. ")


def geometry_shape(geometry):
    from ..geometry import is_volume, is_projection

    if is_volume(geometry):
        return tuple(geometry.shape)
    if is_projection(geometry):
        return (geometry.det_shape[0], geometry.num_angles, geometry.det_shape[1])
    raise ValueError(
        f"Geometry '{type(geometry)}' is not supported. "
        "Cannot determine if volume or projection geometry."
    )


def are_compatible(link_a, link_b):
    """True if both links live on the same device (tomosipo/links/base.py:34-50)."""
    ab = link_a.__compatible_with__(link_b)
    if ab is True:
        return True
    if ab is NotImplemented:
        ba = link_b.__compatible_with__(link_a)
        if ba is True:
            return True
        if ba is NotImplemented:
            warnings.warn(
                f"Cannot determine if link of type {type(link_a)} is compatible with "
                f"{type(link_b)}. Continuing anyway."
            )
            return True
    return False


class Link:
    """Base class of array links."""

    def __init__(self, shape, initial_value):
        self._shape = tuple(shape)

    @staticmethod
    def __accepts__(initial_value):
        raise NotImplementedError()

    def __compatible_with__(self, other):
        raise NotImplementedError()

    @property
    def data(self):
        raise NotImplementedError()

    @data.setter
    def data(self, val):
        raise AttributeError(
            "You cannot change which array backs a dataset.\n"
            "To change the underlying data instead, use: \n"
            " >>> x.data[:] = new_data\n"
        )

    @property
    def shape(self):
        return self._shape

    @contextmanager
    def context(self):
        yield

    def new_zeros(self, shape):
        raise NotImplementedError()

    def new_full(self, shape, value):
        raise NotImplementedError()

    def new_empty(self, shape):
        raise NotImplementedError()

    def clone(self):
        raise NotImplementedError()
