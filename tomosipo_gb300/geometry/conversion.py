"""ASTRA projection-geometry dict -> geometry, under the name tomosipo exposes it
(``tomosipo/geometry/conversion.py:15-30``): ``parallel3d``, ``parallel3d_vec``,
``cone``, ``cone_vec`` and the detector-only ``det_vec`` pseudo-type."""
from .cone import ConeGeometry
from .cone_vec import ConeVectorGeometry
from .det_vec import DetectorVectorGeometry
from .parallel import ParallelGeometry
from .parallel_vec import ParallelVectorGeometry


def from_astra_projection_geometry(astra_pg):
    kinds = {
        "parallel3d": ParallelGeometry,
        "parallel3d_vec": ParallelVectorGeometry,
        "cone": ConeGeometry,
        "cone_vec": ConeVectorGeometry,
        "det_vec": DetectorVectorGeometry,
    }
    kind = astra_pg.get("type")
    if kind not in kinds:
        raise ValueError(f"ASTRA projection geometry type {kind!r} is not supported.")
    return kinds[kind].from_astra(astra_pg)
