"""Host buffers for host <-> device transfers: page-locked and backed by
transparent huge pages.

Host data reaches the GPU by DMA from page-locked memory. On the Grace hosts
of GB300 systems (64 KiB base pages, 512 MiB huge pages, GPU access through
the host's page tables), buffers from ``pin_memory()`` / ``cudaHostAlloc``
sit on base pages; once other processes have come and gone, copies from them
measured occasional stalls of about 25 ms each (a 2.6 ms volume upload took
28 ms, and an end-to-end FP + BP step slowed by up to 40 %), while the same
copies from huge-page buffers in the same state ran at full rate.
``host_buffer`` maps anonymous memory aligned to the huge-page size, asks for
huge pages (``madvise(MADV_HUGEPAGE)``, honoured under the kernel's
``madvise`` transparent-huge-page mode) and registers it with CUDA
(``cudaHostRegister``), so torch sees a pinned tensor and copies are
asynchronous DMA. The mapping is unregistered and unmapped when the last
tensor viewing it is freed.

Where that is not possible (no CUDA device, or a failing system call) the
buffer comes from ``torch.empty(..., pin_memory=True)``, or unpinned memory
without a device: the data path is the same, only the copy rate differs.
"""
import ctypes
import weakref

import numpy as np
import torch

_PROT_READ, _PROT_WRITE = 0x1, 0x2
_MAP_PRIVATE, _MAP_ANONYMOUS = 0x02, 0x20  # Linux (arm64 and x86_64)
_MADV_HUGEPAGE = 14
_MAP_FAILED = ctypes.c_void_p(-1).value

_NUMPY = {torch.float32: np.float32, torch.float64: np.float64, torch.int32: np.int32,
          torch.int64: np.int64, torch.uint8: np.uint8, torch.int16: np.int16,
          torch.float16: np.float16}
_libc = None


def _lib():
    global _libc
    if _libc is None:
        libc = ctypes.CDLL(None, use_errno=True)
        libc.mmap.restype = ctypes.c_void_p
        libc.mmap.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, ctypes.c_long]
        libc.munmap.restype = ctypes.c_int
        libc.munmap.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        libc.madvise.restype = ctypes.c_int
        libc.madvise.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        _libc = libc
    return _libc


def huge_page_bytes():
    """The kernel's transparent huge-page size (2 MiB if it does not say)."""
    try:
        with open("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size") as f:
            return int(f.read())
    except (OSError, ValueError):
        return 2 << 20


def _release(base, length, addr, nbytes, registered):
    if registered:
        torch.cuda.cudart().cudaHostUnregister(addr)
    _lib().munmap(base, length)


def _fallback(shape, dtype):
    if torch.cuda.is_available():
        return torch.empty(shape, dtype=dtype, pin_memory=True)
    return torch.empty(shape, dtype=dtype)


def host_buffer(shape, dtype=torch.float32):
    """Uninitialised page-locked host tensor of ``shape`` on huge pages.

    Use it for the host side of large transfers (``A(x_host)``,
    ``A.T(y_host)``, ``tsgb_copy_sino_angles``). ``tensor.is_pinned()`` is true
    when a CUDA device is present.
    """
    shape = tuple(int(s) for s in (shape if isinstance(shape, (tuple, list, torch.Size))
                                   else (shape,)))
    nbytes = int(np.prod(shape, dtype=np.int64)) * torch.empty((), dtype=dtype).element_size()
    if nbytes == 0 or dtype not in _NUMPY or not torch.cuda.is_available():
        return _fallback(shape, dtype)
    libc = _lib()
    hp = huge_page_bytes()
    span = (nbytes + hp - 1) // hp * hp  # whole huge pages
    length = span + hp  # room to align the start to a huge page
    base = libc.mmap(None, length, _PROT_READ | _PROT_WRITE, _MAP_PRIVATE | _MAP_ANONYMOUS, -1, 0)
    if base in (None, _MAP_FAILED):
        return _fallback(shape, dtype)
    addr = (base + hp - 1) // hp * hp
    libc.madvise(addr, span, _MADV_HUGEPAGE)  # advice only: a refusal leaves base pages
    torch.cuda.init()
    if int(torch.cuda.cudart().cudaHostRegister(addr, nbytes, 0)) != 0:
        libc.munmap(base, length)
        return _fallback(shape, dtype)
    raw = (ctypes.c_byte * nbytes).from_address(addr)
    arr = np.frombuffer(raw, dtype=_NUMPY[dtype]).reshape(shape)
    # the tensor's storage keeps `arr` alive; the mapping goes with it
    fin = weakref.finalize(arr, _release, base, length, addr, nbytes, True)
    fin.atexit = False  # the process's exit releases both
    return torch.from_numpy(arr)
