"""``import tomosipo_gb300.cupy`` (tomosipo: ``import tomosipo.cupy``).

The device-array link that serves CuPy arrays is registered when
``tomosipo_gb300`` is imported (``tomosipo_gb300/links/cuda_array.py``);
this module exists so scripts written for the reference keep working.
"""
from .links.cuda_array import CudaArrayLink  # noqa: F401
