"""Geometry classes with tomosipo's API (``tomosipo/geometry/__init__.py``)."""
from .base_projection import ProjectionGeometry, is_projection, is_cone, is_parallel
from .cone import ConeGeometry, cone, random_cone
from .cone_vec import ConeVectorGeometry, cone_vec, random_cone_vec
from .det_vec import DetectorVectorGeometry, det_vec, random_det_vec
from .parallel import ParallelGeometry, parallel, random_parallel
from .parallel_vec import ParallelVectorGeometry, parallel_vec, random_parallel_vec
from .transform import (
    Transform,
    identity,
    translate,
    scale,
    rotate,
    reflect,
    to_perspective,
    from_perspective,
    random_transform,
)
from .volume import VolumeGeometry, volume, is_volume, random_volume
from .volume_vec import VolumeVectorGeometry, volume_vec, random_volume_vec
from .concatenate import concatenate
from . import conversion
from .conversion import from_astra_projection_geometry
