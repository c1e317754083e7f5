"""``Operator``'s host plumbing on the CPU (tomosipo's ``tests/test_Operator.py``
rules that need no projection): the kernels' entry points are replaced by
fakes that record the call and write a known value, so output allocation,
array-type preservation, ``out=``, ``additive``, ``ts.data`` in and out and the
transpose algebra are checked without a GPU."""
import sys

import numpy as np
import pytest
import torch

import tomosipo_gb300 as ts

# the module, not the class the package exports under the same name
op_module = sys.modules["tomosipo_gb300.Operator"]


@pytest.fixture
def calls(monkeypatch):
    log = []

    def fake_fp(projector, vlink, plink, additive=False):
        log.append(("fp", additive, type(vlink.data), tuple(plink.shape)))
        plink.data[...] = (plink.data if additive else 0) + float(vlink.data.sum())

    def fake_bp(projector, vlink, plink, additive=False, bp_kind="matched"):
        log.append(("bp", additive, bp_kind, tuple(vlink.shape)))
        vlink.data[...] = (vlink.data if additive else 0) + float(plink.data.sum())

    monkeypatch.setattr(op_module, "direct_fp", fake_fp)
    monkeypatch.setattr(op_module, "direct_bp", fake_bp)
    return log


def _geometries():
    return ts.volume(shape=(2, 3, 4)), ts.parallel(angles=5, shape=(2, 6))


@pytest.mark.parametrize("kind", ["numpy", "torch"])
def test_output_type_follows_the_input(calls, kind):
    vg, pg = _geometries()
    A = ts.operator(vg, pg)
    x = np.ones(A.domain_shape, np.float32) if kind == "numpy" else torch.ones(A.domain_shape)
    y = A(x)
    assert type(y) is type(x) and tuple(y.shape) == A.range_shape == (2, 5, 6)
    assert float(y.reshape(-1)[0]) == 24.0
    z = A.T(y)
    assert type(z) is type(x) and tuple(z.shape) == A.domain_shape
    assert [c[0] for c in calls] == ["fp", "bp"]


def test_out_is_written_and_returned(calls):
    vg, pg = _geometries()
    A = ts.operator(vg, pg)
    out = torch.full(A.range_shape, 7.0)
    assert A(torch.ones(A.domain_shape), out=out) is out and float(out[0, 0, 0]) == 24.0


def test_additive_operators_add_into_out_and_start_new_outputs_at_zero(calls):
    vg, pg = _geometries()
    A = ts.operator(vg, pg, additive=True)
    x = torch.ones(A.domain_shape)
    assert float(A(x)[0, 0, 0]) == 24.0  # a new output starts at zero
    out = torch.full(A.range_shape, 1.0)
    A(x, out=out)
    assert float(out[0, 0, 0]) == 25.0 and all(c[1] for c in calls)


def test_datasets_in_give_datasets_out_on_the_operators_geometry(calls):
    vg, pg = _geometries()
    A = ts.operator(vg, pg)
    vd = ts.data(vg, 1.0)
    pd = A(vd)
    assert isinstance(pd, ts.Data.Data) and pd.geometry == pg and float(pd.data[0, 0, 0]) == 24.0
    vd2 = A.T(pd)
    assert isinstance(vd2, ts.Data.Data) and vd2.geometry == vg


def test_backprojector_choice_reaches_the_kernel_call(calls):
    vg, pg = _geometries()
    for kind in ("matched", "bilinear"):
        ts.operator(vg, pg, backprojector=kind).T(torch.ones(2, 5, 6))
    assert [c[2] for c in calls] == ["matched", "bilinear"]
    with pytest.raises(ValueError):
        ts.operator(vg, pg, backprojector="nearest")


def test_transpose_algebra():
    vg, pg = _geometries()
    A = ts.operator(vg, pg)
    assert A.T.T is A and A.T.T.T is A.T
    assert A.T.domain == A.range == pg and A.T.range == A.domain == vg
    assert A.T.domain_shape == A.range_shape and A.T.range_shape == A.domain_shape
