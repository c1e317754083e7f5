"""Thread-to-voxel maps of the backprojection kernels, restated on the host.

``bp_separable_kernel`` (``tomosipo_gb300/csrc/bp.cu``): a block of 128 threads
is kTA threads along the in-plane axis a times 128 / kTA planes, a-fastest or
plane-fastest (kPF, which also swaps the grid's x and y); each thread owns
kA = 2 voxels along a and kRun = 16 along z. ``bp_bilinear_z_kernel``: kTX
voxel columns along x times 128 / kTX along y, 16 voxels along z.
``bp_weight_kernel``: a thread writes 8 consecutive row pairs of one detector
column, from row -1. These restatements must cover every voxel (or row) exactly
once for ragged sizes, with every write inside the buffer; the GPU tests check
the values.
"""
import itertools

import numpy as np
import pytest

THREADS, KA, KRUN = 128, 2, 16


def separable_cover(n_a, n_p, nz, kta, kpf):
    """Counts of writes per voxel (a, plane, z) of one pass's launch."""
    ktp = THREADS // kta
    ga = -(-n_a // (kta * KA))
    gp = -(-n_p // ktp)
    gz = -(-nz // KRUN)
    grid_x, grid_y = (gp, ga) if kpf else (ga, gp)
    hits = np.zeros((n_a, n_p, nz), dtype=np.int32)
    for bx, by, bz in itertools.product(range(grid_x), range(grid_y), range(gz)):
        ba, bp = (by, bx) if kpf else (bx, by)
        for t in range(THREADS):
            ta, tp = (t // ktp, t % ktp) if kpf else (t % kta, t // kta)
            ia0, ip, z0 = (ba * kta + ta) * KA, bp * ktp + tp, bz * KRUN
            if ia0 >= n_a or ip >= n_p:
                continue  # the kernel returns before any write
            for m, j in itertools.product(range(KA), range(KRUN)):
                if ia0 + m < n_a and z0 + j < nz:  # the epilogue's own tests
                    hits[ia0 + m, ip, z0 + j] += 1
    return hits


@pytest.mark.parametrize("kta, kpf", [(8, False), (4, True), (32, False), (16, True)])
@pytest.mark.parametrize("n_a, n_p, nz", [(33, 20, 17), (64, 64, 32), (7, 130, 5), (1, 1, 1)])
def test_separable_tiles_cover_every_voxel_once(kta, kpf, n_a, n_p, nz):
    assert np.all(separable_cover(n_a, n_p, nz, kta, kpf) == 1)


def bilinear_cover(nx, ny, nz, ktx):
    kty = THREADS // ktx
    hits = np.zeros((nx, ny, nz), dtype=np.int32)
    for bx, by, bz in itertools.product(range(-(-nx // ktx)), range(-(-ny // kty)),
                                        range(-(-nz // KRUN))):
        for t in range(THREADS):
            x, y = bx * ktx + t % ktx, by * kty + t // ktx
            if x >= nx or y >= ny:
                continue
            for j in range(KRUN):
                if bz * KRUN + j < nz:
                    hits[x, y, bz * KRUN + j] += 1
    return hits


@pytest.mark.parametrize("ktx", [8, 32])
@pytest.mark.parametrize("shape", [(37, 20, 17), (8, 4, 16), (1, 1, 1)])
def test_bilinear_tiles_cover_every_voxel_once(ktx, shape):
    assert np.all(bilinear_cover(*shape, ktx) == 1)


@pytest.mark.parametrize("rows", [1, 7, 8, 63, 64, 65, 512])
def test_weight_pass_writes_each_row_pair_once(rows):
    """Pair rows -1 .. rows-1 are written once each, and each reads detector
    rows r and r + 1 (zero outside 0 .. rows-1), never past the padding."""
    per_thread, threads_y = 8, 8
    grid_y = -(-(rows + 1) // (threads_y * per_thread))
    written = []
    for by, ty in itertools.product(range(grid_y), range(threads_y)):
        r0 = (by * threads_y + ty) * per_thread - 1
        if r0 >= rows:
            continue
        written += [r0 + k for k in range(per_thread) if r0 + k < rows]
    assert sorted(written) == list(range(-1, rows))
    pad_rows = 2  # rows -2 .. rows + 1 exist in the workspace
    assert min(written) >= -pad_rows and max(written) + 1 <= rows + pad_rows - 1
