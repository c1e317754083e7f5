from .base import link, geometry_shape, are_compatible, Link, backends
from .numpy import NumpyLink

try:
    from .torch import TorchLink
    from .cuda_array import CudaArrayLink
except ImportError:  # torch missing: NumPy links only
    TorchLink = CudaArrayLink = None
