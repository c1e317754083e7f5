"""Device-array link (the role of tomosipo's CuPy link): objects exposing
__cuda_array_interface__ project in place, zero copy. CuPy is not installed
here, so a minimal stand-in array type carries the interface."""
import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300.links import CudaArrayLink

torch = pytest.importorskip("torch")


class DeviceArray:
    """Exposes another tensor's memory through the CUDA array interface only."""

    def __init__(self, t):
        self._t = t
        self.__cuda_array_interface__ = t.__cuda_array_interface__
        self.shape = tuple(t.shape)


def test_accepts_only_interface_objects():
    class Fake:
        __cuda_array_interface__ = {}

    assert CudaArrayLink.__accepts__(Fake())
    assert not CudaArrayLink.__accepts__(np.zeros(3))
    assert not CudaArrayLink.__accepts__(torch.zeros(3))
    import tomosipo_gb300.cupy  # noqa: F401  (the reference's import still works)
    from tomosipo_gb300.links.cupy import CupyLink  # and its link module's name

    assert CupyLink is CudaArrayLink


@pytest.mark.gpu
def test_projects_in_place_through_the_interface(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda", 0)
    vg = ts.volume(shape=16, size=1)
    pg = ts.cone(angles=8, shape=(16, 24), size=1.5, cone_angle=0.4)
    A = ts.operator(vg, pg)
    x = torch.rand(A.domain_shape, device=dev)
    y_ref = A(x)
    y = A(DeviceArray(x))  # a new output: a torch tensor without CuPy
    assert torch.equal(torch.as_tensor(y), y_ref)
    out = torch.zeros(A.range_shape, device=dev)
    A(DeviceArray(x), out=DeviceArray(out))  # written in place, zero copy
    assert torch.equal(out, y_ref)
    back = torch.zeros(A.domain_shape, device=dev)
    A.T(DeviceArray(out), out=DeviceArray(back))
    assert torch.equal(back, A.T(y_ref))
    with pytest.warns(UserWarning):
        A(DeviceArray(x.double()))
