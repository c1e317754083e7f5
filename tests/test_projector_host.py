"""The link layer's host-side checks (``tomosipo_gb300.projector.direct_project``,
after ``tomosipo/astra.py:104-153``), which run before any CUDA call, and the
absence of a CPU fallback: without a CUDA device a projection raises."""
import numpy as np
import pytest
import torch

import tomosipo_gb300 as ts
from tomosipo_gb300 import projector as P


def _setup():
    vg, pg = ts.volume(shape=(2, 3, 4)), ts.parallel(angles=5, shape=(2, 6))
    vol = ts.link(vg, np.zeros((2, 3, 4), np.float32))
    sino = ts.link(pg, np.zeros((2, 5, 6), np.float32))
    return vg, pg, vol, sino


def test_direction_must_be_given():
    vg, pg, vol, sino = _setup()
    with pytest.raises(ValueError, match="forward argument"):
        P.direct_project(P.create_projector(vg, pg), vol, sino, forward=None)


def test_unknown_backprojector_is_rejected():
    vg, pg, vol, sino = _setup()
    with pytest.raises(ValueError, match="bp_kind"):
        P.direct_project(P.create_projector(vg, pg), vol, sino, forward=False, bp_kind="nearest")


def test_links_must_match_the_projectors_shapes():
    vg, pg, vol, sino = _setup()
    other = P.create_projector(ts.volume(shape=(2, 3, 5)), pg)
    with pytest.raises(ValueError, match=r"Expected volume \(2, 3, 5\)"):
        P.direct_project(other, vol, sino, forward=True)


def test_projectors_need_ray_geometries_and_valid_factors():
    vg, pg, _, _ = _setup()
    with pytest.raises(TypeError):
        P.create_projector(vg, ts.volume(shape=3))
    with pytest.raises(TypeError):
        P.create_projector(vg.to_vec(), pg)
    with pytest.raises(ValueError):
        P.create_projector(vg, pg, detector_supersampling=0)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_no_cpu_fallback_without_a_gpu():
    vg, pg, vol, sino = _setup()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        P.direct_project(P.create_projector(vg, pg), vol, sino, forward=True)
    A = ts.operator(vg, pg)
    for x in (np.zeros(A.domain_shape, np.float32), torch.zeros(A.domain_shape)):
        with pytest.raises(RuntimeError, match="CUDA GPU only"):
            A(x)
