"""tomosipo_gb300: tomosipo's operator API on hand-written sm_103a CUDA kernels.

``import tomosipo_gb300 as ts`` gives the names tomosipo exports for the
projection path (``tomosipo/__init__.py:10-41``): ``operator``, ``data``,
``volume``, ``volume_vec``, ``parallel``, ``parallel_vec``, ``cone``,
``cone_vec``, the transforms, ``concatenate``, ``link``, ``to_astra`` /
``from_astra`` and ``epsilon``; ``tomosipo_gb300.astra`` has the legacy ``forward``/``backward``
and ``fdk``.
"""
__version__ = "0.6.0+gb300"

from .Operator import operator, Operator, BackprojectionOperator
from .Data import data
from .geometry.volume import volume
from .geometry.volume_vec import volume_vec
from . import geometry
from .geometry.cone import cone
from .geometry.cone_vec import cone_vec
from .geometry.parallel_vec import parallel_vec
from .geometry.parallel import parallel
from .geometry.transform import (
    translate,
    scale,
    rotate,
    reflect,
    to_perspective,
    from_perspective,
)
from .geometry.concatenate import concatenate
from .links.base import link
from . import links
from . import phantom
from . import types
from . import vector_calc
from .hostmem import host_buffer

# Used for floating-point equality checks and the SIRT clipping 1 / epsilon
# (tomosipo/__init__.py:41).
epsilon = 1e-8


def to_astra(x):
    """ASTRA geometry dict of a tomosipo geometry (tomosipo/astra.py:56-77)."""
    try:
        return x.to_astra()
    except AttributeError:
        raise TypeError(
            f"The object of type {type(x)} does not support conversion to ASTRA."
            "Perhaps you meant to use `ts.from_astra'? "
        )


def from_astra(astra_geom):
    """Geometry from an ASTRA 3D geometry dict (tomosipo/astra.py:35-53)."""
    if not isinstance(astra_geom, dict):
        raise TypeError(
            "Currently, tomosipo only supports importing ASTRA geometries. "
            f"Objects of type {type(astra_geom)} are not supported. "
            "Perhaps you meant to use `ts.to_astra'? "
        )
    if "GridSliceCount" in astra_geom:
        from .geometry.volume import from_astra as volume_from_astra

        return volume_from_astra(astra_geom)
    return geometry.from_astra_projection_geometry(astra_geom)
