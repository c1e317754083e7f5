"""Managed datasets for the legacy projection functions (``tomosipo/Data.py``).

``data(geometry, initial_value=None)`` pairs an ASTRA-compatible geometry (an
axis-aligned ``volume``, or a ``parallel``/``cone``/``*_vec`` projection
geometry) with an array link, as tomosipo's ``Data`` does. Here the array is
not registered with ASTRA: ``tomosipo_gb300.astra.forward``/``backward``/
``fdk`` project between datasets with this package's kernels. Behaviour kept
from the reference (``tomosipo/Data.py:6-152``): ``initial_value`` may be
``None`` (zeros), a scalar, a NumPy array or a torch tensor (NumPy arrays and
CPU/GPU tensors are shared, not copied, when they already are contiguous
float32); passing a ``Data`` with the same geometry returns it; geometries
without an ASTRA form raise ``TypeError``; ``with ts.data(...) as d`` works.
"""
from .geometry import is_projection, is_volume
from .links.base import link


def data(geometry, initial_value=None):
    """Dataset for ``geometry`` (``tomosipo/Data.py:6-29``)."""
    if isinstance(initial_value, Data):
        if geometry == initial_value.geometry:
            return initial_value
        raise ValueError(
            f"Got initial_value={initial_value}, "
            f"but its geometry does not match {geometry}."
        )
    return Data(geometry, initial_value)


class Data:
    """A geometry plus the array that holds its values."""

    def __init__(self, geometry, initial_value=None):
        self.geometry = geometry
        if not hasattr(geometry, "to_astra"):
            raise TypeError(
                "Cannot create data object with geometry because it is not convertible to "
                f"ASTRA: {geometry}"
            )
        if not (self.is_volume() or self.is_projection()):
            raise ValueError(
                f"Geometry '{type(geometry)}' is not supported. Cannot determine if volume "
                "or projection geometry."
            )
        self._link = link(geometry, initial_value)

    def clone(self):
        """A new dataset with the same geometry and a copy of the values."""
        return Data(self.geometry, self._link.clone().data)

    def __enter__(self):
        return self

    def __exit__(self, type, value, traceback):
        return None

    @property
    def data(self):
        """The underlying array (projection data is ordered (V, num_angles, U))."""
        return self._link.data

    @data.setter
    def data(self, val):
        self._link.data = val

    @property
    def link(self):
        return self._link

    def is_volume(self):
        return is_volume(self.geometry)

    def is_projection(self):
        return is_projection(self.geometry)

    def __repr__(self):
        return f"Data(\n    geometry={self.geometry},\n    data=<{type(self.data)} of shape {self._link.shape}>\n)"
