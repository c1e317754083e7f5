"""The C-ABI library: it loads, exports every declared entry point, and rejects
bad geometry on the host before any CUDA call (no GPU needed)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import tomosipo_gb300 as ts
from tomosipo_gb300 import _build, _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    _build.build_library()
    return _native.load()


def declared_functions():
    names = set()
    for header in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(header).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(tsgb_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def exported_symbols(path):
    import subprocess

    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "tsgb_direct_fp" in names and "tsgb_direct_bp" in names
    exported = exported_symbols(_build.LIBPATH)
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def test_bindings_cover_every_declaration():
    assert set(declared_functions()) == set(_native.SIGNATURES)


def _descs(vec, kind=_native.TSGB_CONE, shape=(8, 8, 8), det=(4, 5)):
    v = _native.VolumeDesc()
    v.shape[:] = list(shape)
    v.pos[:] = [0, 0, 0]
    v.size[:] = [1, 1, 1]
    p = _native.ProjectionDesc()
    p.kind = kind
    p.det_shape[:] = list(det)
    vec = np.ascontiguousarray(vec, dtype=np.float64)
    p.num_angles = vec.shape[0]
    p.vectors = vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return v, p, vec


def _create(lib, v, p, vss=1, dss=1):
    out = ctypes.c_void_p()
    rc = lib.tsgb_projector_create(ctypes.byref(v), ctypes.byref(p), vss, dss, ctypes.byref(out))
    return rc, out


GOOD = np.array([[0, -3, 0, 0, 1, 0, 0.1, 0, 0, 0, 0, 0.1]], dtype=np.float64)


@pytest.mark.parametrize(
    "mutate,msg",
    [
        (lambda v, p, a: a.__setitem__((0, 0), np.nan), "non-finite"),
        (lambda v, p, a: a.__setitem__((0, slice(9, 12)), 0.0), "degenerate"),
        (lambda v, p, a: setattr(p, "kind", 7), "kind"),
        (lambda v, p, a: v.shape.__setitem__(0, 0), "volume shape"),
        (lambda v, p, a: v.size.__setitem__(1, -1.0), "size"),
        (lambda v, p, a: p.det_shape.__setitem__(1, 0), "detector shape"),
        (lambda v, p, a: setattr(p, "num_angles", 0), "angles"),
    ],
)
def test_invalid_geometry_is_rejected_on_host(lib, mutate, msg):
    v, p, vec = _descs(GOOD.copy())
    mutate(v, p, vec)
    rc, out = _create(lib, v, p)
    assert rc == -1
    assert out.value is None
    assert msg in lib.tsgb_last_error().decode()


def test_bad_supersampling_is_rejected(lib):
    v, p, vec = _descs(GOOD.copy())
    assert _create(lib, v, p, vss=0)[0] == -1
    assert _create(lib, v, p, dss=17)[0] == -1


def test_null_arguments(lib):
    assert lib.tsgb_projector_create(None, None, 1, 1, None) == -1
    assert lib.tsgb_direct_fp(None, None, None, 0, None, 0, None) == -1
    assert lib.tsgb_direct_bp(None, None, None, 0, 0, None, 0, None) == -1
    assert lib.tsgb_projector_destroy(None) == 0


def test_projection_vectors_layout():
    from tomosipo_gb300.projector import projection_vectors

    pg = ts.cone(angles=3, shape=(4, 5), size=(1, 2), src_orig_dist=3, src_det_dist=4)
    kind, rows, cols, vec = projection_vectors(pg)
    pv = pg.to_vec()
    assert kind == _native.TSGB_CONE and (rows, cols) == (4, 5)
    assert np.allclose(vec[:, 0:3], pv.src_pos)
    assert np.allclose(vec[:, 3:6], pv.det_pos)
    assert np.allclose(vec[:, 6:9], pv.det_v)
    assert np.allclose(vec[:, 9:12], pv.det_u)


# Every other entry point: NULL handles or pointers are rejected with -1 and a
# message before any CUDA call; destroying NULL is a no-op.
_NULL_CALLS = {
    "tsgb_fp_workspace_bytes": (None,),
    "tsgb_bp_workspace_bytes": (None, 0),
    "tsgb_bp_batch_workspace_bytes": (None, 2, 0),
    "tsgb_fp_batch_workspace_bytes": (None, 2),
    "tsgb_projector_shapes": (None, None, None),
    "tsgb_projector_stats": (None, None, 8),
    "tsgb_projector_get_tuning": (None, None),
    "tsgb_projector_set_tuning": (None, None),
    "tsgb_direct_fp_batch": (None, None, None, 2, 0, None, 0, None),
    "tsgb_direct_bp_batch": (None, None, None, 2, 0, 0, None, 0, None),
    "tsgb_direct_fp_angles": (None, None, None, 0, 0, 1, 0, None, 0, None),
    "tsgb_direct_bp_angles": (None, None, None, 0, 0, 1, None, 0, None),
    "tsgb_copy_sino_angles": (None, None, 1, 1, 1, 0, 1, None),
    "tsgb_fdk_backproject": (None, None, None, None, 0, None, 0, None),
    "tsgb_direct_fp_noalloc": (None, None, None, None, 0, None),
    "tsgb_sirt_batch_create": (None, 0, None),
    "tsgb_sirt_batch_iterate": (None, 1, None),
    "tsgb_sirt_batch_iterate_jobs": (None, None, None),
}


@pytest.mark.parametrize("name", sorted(_NULL_CALLS))
def test_null_arguments_of_every_entry_point(lib, name):
    assert getattr(lib, name)(*_NULL_CALLS[name]) == -1
    assert lib.tsgb_last_error().decode()
    assert lib.tsgb_sirt_batch_destroy(None) == 0


def test_null_cases_cover_the_declarations():
    covered = set(_NULL_CALLS) | {"tsgb_projector_create", "tsgb_direct_fp", "tsgb_direct_bp",
                                  "tsgb_projector_destroy", "tsgb_sirt_batch_destroy",
                                  "tsgb_last_error"}
    assert covered == set(declared_functions())
