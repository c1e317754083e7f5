"""Build the native projector library (and the CPU oracle) in-tree.

``libtomosipo_gb300.so`` is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), one translation unit per
process, and linked with the static CUDA runtime. Output goes to
``tomosipo_gb300/_lib/``; nothing is installed into site-packages.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "_lib")
LIBNAME = "libtomosipo_gb300.so"
LIBPATH = os.path.join(LIBDIR, LIBNAME)

CUDA_SOURCES = ["fp.cu", "bp.cu", "bp_zlane.cu", "capi.cu", "batch.cu", "noalloc.cu", "supersample.cu"]
CXX_SOURCES = ["plan.cpp"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tomosipo_gb300")


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return proc.stdout


def _sources():
    return [s for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))], CXX_SOURCES


def _newest_input_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "tomosipo_gb300.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def build_library(force=False, verbose=False):
    """Compile csrc/*.cu and csrc/*.cpp into tomosipo_gb300/_lib/libtomosipo_gb300.so."""
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= _newest_input_mtime():
        return LIBPATH
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    cu, cxx = _sources()
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
    jobs = []
    for src in cu:
        obj = os.path.join(objdir, src + ".o")
        jobs.append([nvcc, *GENCODE, *flags, "-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o", obj])
    for src in cxx:
        obj = os.path.join(objdir, src + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-I", CSRC,
                     "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    objs = [os.path.join(objdir, s + ".o") for s in cu + cxx]
    tmp = LIBPATH + ".tmp"
    _run([nvcc, *GENCODE, "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs])
    os.replace(tmp, LIBPATH)
    return LIBPATH


ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")


def build_oracle(force=False):
    """Compile the FP64 CPU oracle (test infrastructure) into oracle/liboracle.so."""
    src = os.path.join(ORACLE_DIR, "oracle.cpp")
    hdr = os.path.join(INCLUDE, "tomosipo_gb300.h")
    newest = max(os.path.getmtime(src), os.path.getmtime(hdr))
    if not force and os.path.exists(ORACLE_LIB) and os.path.getmtime(ORACLE_LIB) >= newest:
        return ORACLE_LIB
    tmp = ORACLE_LIB + ".tmp"
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-I", INCLUDE,
          src, "-o", tmp])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
    print(build_oracle(force="--force" in sys.argv))
