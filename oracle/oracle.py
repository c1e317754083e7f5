"""ctypes wrapper of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/ and ``__graft_entry__.smoke()`` as the values the GPU results
are compared with, and by the CPU-baseline leg of ``bench.py`` as the timed CPU
baseline; never by the product path. The arithmetic lives in ``oracle.cpp``;
this file only converts tomosipo geometry objects to the C descriptors (volume
shape/pos/size and the vector rows ``[src_pos or ray_dir, det_pos, det_v,
det_u]`` in (z, y, x)).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
_lib = None


class _Vol(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_int64 * 3), ("pos", ctypes.c_double * 3),
                ("size", ctypes.c_double * 3)]


class _Proj(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("det_shape", ctypes.c_int64 * 2), ("num_angles", ctypes.c_int64),
                ("vectors", ctypes.POINTER(ctypes.c_double))]


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            import sys
            sys.path.insert(0, os.path.dirname(HERE))
            from tomosipo_gb300._build import build_oracle
            build_oracle()
        lib = ctypes.CDLL(LIB)
        for name in ("oracle_fp", "oracle_bp_matched", "oracle_bp_bilinear"):
            fn = getattr(lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.POINTER(_Vol), ctypes.POINTER(_Proj), ctypes.c_int,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib = lib
    return _lib


def descriptors(vg, pg):
    """C descriptors for an axis-aligned volume and a projection geometry."""
    v = _Vol()
    v.shape[:] = list(vg.shape)
    v.pos[:] = [float(x) for x in np.asarray(vg.pos).reshape(-1)[:3]]
    v.size[:] = [float(x) for x in vg.size]
    pv = pg.to_vec()
    first = pv.src_pos if pg.is_cone else pv.ray_dir
    vec = np.ascontiguousarray(
        np.concatenate([first, pv.det_pos, pv.det_v, pv.det_u], axis=1), dtype=np.float64)
    p = _Proj()
    p.kind = 1 if pg.is_cone else 0
    p.det_shape[:] = list(pv.det_shape)
    p.num_angles = vec.shape[0]
    p.vectors = vec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return v, p, vec


def _threads(n):
    return int(n) if n else max(1, os.cpu_count() or 1)


def _sino_shape(pg):
    return (pg.det_shape[0], pg.num_angles, pg.det_shape[1])


def fp(vg, pg, vol, det_ss=1, threads=None):
    """Forward projection (rows, angles, cols) in float64."""
    v, p, _keep = descriptors(vg, pg)
    x = np.ascontiguousarray(vol, dtype=np.float64)
    assert x.shape == tuple(vg.shape)
    y = np.zeros(_sino_shape(pg), dtype=np.float64)
    rc = load().oracle_fp(ctypes.byref(v), ctypes.byref(p), det_ss, x.ctypes.data, y.ctypes.data,
                          _threads(threads))
    if rc:
        raise ValueError("oracle_fp rejected its arguments")
    return y


def bp_matched(vg, pg, sino, det_ss=1, threads=None):
    """Exact transpose of ``fp`` (z, y, x) in float64."""
    v, p, _keep = descriptors(vg, pg)
    y = np.ascontiguousarray(sino, dtype=np.float64)
    assert y.shape == _sino_shape(pg)
    x = np.zeros(tuple(vg.shape), dtype=np.float64)
    rc = load().oracle_bp_matched(ctypes.byref(v), ctypes.byref(p), det_ss, y.ctypes.data,
                                  x.ctypes.data, _threads(threads))
    if rc:
        raise ValueError("oracle_bp_matched rejected its arguments")
    return x


def bp_bilinear(vg, pg, sino, vox_ss=1, threads=None):
    """Voxel-driven bilinear backprojection (z, y, x) in float64."""
    v, p, _keep = descriptors(vg, pg)
    y = np.ascontiguousarray(sino, dtype=np.float64)
    assert y.shape == _sino_shape(pg)
    x = np.zeros(tuple(vg.shape), dtype=np.float64)
    rc = load().oracle_bp_bilinear(ctypes.byref(v), ctypes.byref(p), vox_ss, y.ctypes.data,
                                   x.ctypes.data, _threads(threads))
    if rc:
        raise ValueError("oracle_bp_bilinear rejected its arguments")
    return x
