"""ctypes binding of ``libtomosipo_gb300.so`` (the C ABI in include/tomosipo_gb300.h).

This is the only route to the projection kernels. There is no CPU or
PyTorch fallback: if the library has not been built, every projection
raises ``RuntimeError``.
"""
import ctypes
import os
import threading

from ._build import LIBPATH

TSGB_OK = 0
TSGB_PARALLEL = 0
TSGB_CONE = 1
TSGB_BP_MATCHED = 0
TSGB_BP_BILINEAR = 1

c_int64_3 = ctypes.c_int64 * 3
c_double_3 = ctypes.c_double * 3


class VolumeDesc(ctypes.Structure):
    _fields_ = [("shape", c_int64_3), ("pos", c_double_3), ("size", c_double_3)]


class ProjectionDesc(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("det_shape", ctypes.c_int64 * 2),
        ("num_angles", ctypes.c_int64),
        ("vectors", ctypes.POINTER(ctypes.c_double)),
    ]


class SirtJob(ctypes.Structure):
    _fields_ = [
        ("projector", ctypes.c_void_p),
        ("vol", ctypes.c_void_p),
        ("sino", ctypes.c_void_p),
        ("R", ctypes.c_void_p),
        ("C", ctypes.c_void_p),
        ("residual", ctypes.c_void_p),
        ("fp_workspace", ctypes.c_void_p),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [
        ("fp_patch_rows", ctypes.c_int32),
        ("fp_patch_cols", ctypes.c_int32),
        ("fp_group_pairs", ctypes.c_int32),
        ("fp_pair_layout", ctypes.c_int32),
        ("bp_kernel", ctypes.c_int32),
        ("bp_shape", ctypes.c_int32),
        ("bp_general", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


_lib = None
_lock = threading.Lock()

# name -> (restype, argtypes)
SIGNATURES = {
    "tsgb_projector_create": (
        ctypes.c_int,
        [ctypes.POINTER(VolumeDesc), ctypes.POINTER(ProjectionDesc), ctypes.c_int32,
         ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)],
    ),
    "tsgb_projector_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tsgb_fp_workspace_bytes": (ctypes.c_int64, [ctypes.c_void_p]),
    "tsgb_bp_workspace_bytes": (ctypes.c_int64, [ctypes.c_void_p, ctypes.c_int32]),
    "tsgb_bp_batch_workspace_bytes": (ctypes.c_int64, [ctypes.c_void_p, ctypes.c_int64,
                                                       ctypes.c_int32]),
    "tsgb_fp_batch_workspace_bytes": (ctypes.c_int64, [ctypes.c_void_p, ctypes.c_int64]),
    "tsgb_direct_fp": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
         ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_direct_bp": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_projector_shapes": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    ),
    "tsgb_projector_stats": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_int32]
    ),
    "tsgb_direct_fp_noalloc": (
        ctypes.c_int,
        [ctypes.POINTER(VolumeDesc), ctypes.POINTER(ProjectionDesc), ctypes.c_void_p,
         ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p],
    ),
    "tsgb_sirt_batch_create": (
        ctypes.c_int, [ctypes.POINTER(SirtJob), ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]
    ),
    "tsgb_sirt_batch_iterate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "tsgb_sirt_batch_iterate_jobs": (
        ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]
    ),
    "tsgb_sirt_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tsgb_projector_get_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tuning)]),
    "tsgb_projector_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tuning)]),
    "tsgb_direct_fp_batch": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_direct_bp_batch": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
         ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_direct_fp_angles": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64,
         ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_direct_bp_angles": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64,
         ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_copy_sino_angles": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
         ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_fdk_backproject": (
        ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
         ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p],
    ),
    "tsgb_last_error": (ctypes.c_char_p, []),
}


def library_path():
    return LIBPATH


def load():
    """Load the native library (once). Raises RuntimeError if it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIBPATH):
            raise RuntimeError(
                f"tomosipo_gb300 native library not found at {LIBPATH}. "
                "Build it first: python -c 'import __graft_entry__ as g; g.build()' "
                "(or python -m tomosipo_gb300._build)."
            )
        lib = ctypes.CDLL(LIBPATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return _lib


def check(rc, what):
    if rc != TSGB_OK:
        msg = load().tsgb_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed (code {rc}): {msg}")
