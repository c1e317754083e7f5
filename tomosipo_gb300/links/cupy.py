"""``tomosipo_gb300.links.cupy`` (tomosipo: ``tomosipo/links/cupy.py``).

CuPy arrays are served by the device-array link (any object with
``__cuda_array_interface__``), registered when ``tomosipo_gb300`` is
imported; ``CupyLink`` is that link under the reference's name.
"""
from .cuda_array import CudaArrayLink as CupyLink  # noqa: F401
