"""``ts.concatenate``: join geometries or transforms along their step axis.

The documented behaviour of tomosipo's ``concatenate``
(``tomosipo/geometry/concatenate.py:16-88``): a sequence of transforms gives
one transform with all their steps; parallel geometries (vector or not)
give a ``parallel_vec``, cone geometries a ``cone_vec`` and volumes a
``volume_vec``, each holding the steps of the items in order. Projection
geometries must share their detector shape and volumes their shape
(``ValueError`` otherwise); an empty sequence is a ``ValueError``, a bare
geometry instead of a sequence and a mix of kinds are ``TypeError``s.
"""
import numpy as np

from .base_projection import ProjectionGeometry, is_cone, is_parallel
from .cone_vec import cone_vec
from .parallel_vec import parallel_vec
from .transform import Transform
from .volume import VolumeGeometry, is_volume
from .volume_vec import VolumeVectorGeometry, volume_vec


def _stack(items, name):
    return np.concatenate([np.asarray(getattr(i, name), dtype=np.float64) for i in items])


def concatenate(items):
    """One geometry (or transform) with the steps of ``items`` in order."""
    if isinstance(items, (ProjectionGeometry, VolumeGeometry, VolumeVectorGeometry, Transform)):
        raise TypeError("items must be a sequence of geometries or transforms. ")
    items = list(items)
    if len(items) == 0:
        raise ValueError("ts.concatenate expected at least one argument. ")
    if all(isinstance(i, Transform) for i in items):
        return Transform(np.concatenate([i.matrix for i in items]))
    if all(is_parallel(i) for i in items) or all(is_cone(i) for i in items):
        shape = items[0].det_shape
        if any(i.det_shape != shape for i in items):
            raise ValueError("Cannot concatenate geometries. Not all detector shapes are equal.")
        common = dict(shape=shape, det_pos=_stack(items, "det_pos"),
                      det_v=_stack(items, "det_v"), det_u=_stack(items, "det_u"))
        if is_parallel(items[0]):
            return parallel_vec(ray_dir=_stack(items, "ray_dir"), **common)
        return cone_vec(src_pos=_stack(items, "src_pos"), **common)
    if all(is_volume(i) for i in items):
        shape = tuple(items[0].shape)
        if any(tuple(i.shape) != shape for i in items):
            raise ValueError("Cannot concatenate volumes. Not all shapes are equal.")
        return volume_vec(shape=shape, pos=_stack(items, "pos"), w=_stack(items, "w"),
                          v=_stack(items, "v"), u=_stack(items, "u"))
    kinds = sorted({type(i).__name__ for i in items})
    raise TypeError(f"Concatenating objects of types {kinds} is not supported. ")
