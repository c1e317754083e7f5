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


# ---------------------------------------------------------------- z-lane kernels
# bp_zlane_kernel (tomosipo_gb300/csrc/bp_zlane.cu): a block is kPlanes warps on
# adjacent planes; blockIdx.x = window * plane_blocks + plane block, blockIdx.y
# = z range; lane l of a warp owns the kX voxels i0 .. i0 + kX - 1 along a and
# z = z0 + l + 32 j for j < kRun. Its stores go to the [y][x][z] scratch volume.
ZLANE_SHAPES = [(4, 8, 4), (4, 8, 8), (4, 16, 8), (4, 16, 16), (3, 16, 8), (4, 4, 4), (4, 2, 4)]


def zlane_cover(nx, ny, nz, kx, krun, kplanes, a_is_x):
    """Write counts per scratch element [y][x][z] of one pass's launch."""
    n_p, n_a = (ny, nx) if a_is_x else (nx, ny)
    plane_blocks = -(-n_p // kplanes)
    windows = -(-n_a // kx)
    gz = -(-nz // (32 * krun))
    hits = np.zeros(ny * nx * nz, dtype=np.int32)
    for bx, by in itertools.product(range(plane_blocks * windows), range(gz)):
        pb, wb = bx % plane_blocks, bx // plane_blocks
        for w, lane in itertools.product(range(kplanes), range(32)):
            ip, i0 = pb * kplanes + w, wb * kx
            if ip >= n_p:
                continue  # the warp returns before any access
            z0 = by * 32 * krun + lane
            for m in range(kx):
                ia = i0 + m
                if ia >= n_a:
                    break
                base = (ip * nx + ia) * nz if a_is_x else (ia * nx + ip) * nz
                for j in range(krun):
                    z = z0 + 32 * j
                    if z < nz:
                        assert 0 <= base + z < hits.size
                        hits[base + z] += 1
    return hits


@pytest.mark.parametrize("shape", ZLANE_SHAPES)
@pytest.mark.parametrize("dims", [(9, 13, 70), (4, 4, 1), (33, 5, 257), (1, 1, 1)])
@pytest.mark.parametrize("a_is_x", [True, False])
def test_zlane_tiles_cover_every_voxel_once(shape, dims, a_is_x):
    assert np.all(zlane_cover(*dims, *shape, a_is_x) == 1)


@pytest.mark.parametrize("rows, cols", [(1, 1), (7, 40), (32, 32), (62, 65), (512, 768)])
def test_weight_z_pass_writes_each_padded_pair_once(rows, cols):
    """bp_weight_z_kernel: blocks of 32 columns x 32 padded pair rows of one
    angle; every padded pair (theta, iu, r), r < rows + 4, is written once, from
    shared-memory rows r and r + 1 of its block's 33 (detector rows
    r0 + k - 2, zero off the detector)."""
    RP = rows + 4
    hits = np.zeros((cols, RP), dtype=np.int32)
    for bx, by in itertools.product(range(-(-cols // 32)), range(-(-RP // 32))):
        r0 = by * 32
        for tx, ty in itertools.product(range(32), range(8)):
            r = r0 + tx
            if r >= RP:
                continue
            for c in range(ty, 32, 8):
                iu = bx * 32 + c
                if iu >= cols:
                    break
                assert tx + 1 < 33  # shared rows read
                hits[iu, r] += 1
    assert np.all(hits == 1)


@pytest.mark.parametrize("rows", [1, 2, 5, 64, 511, 512])
def test_zlane_row_reads_stay_in_the_padded_column(rows):
    """The fast loop reads anchored rows floor(t) for t in [vmin, vmax + 1) and
    the clamped loop clamps t to [vmin, vmax]: with vmin = -2 - rows // 2 and
    vmax = rows - rows // 2, every pair index (2 + rows // 2 + floor(t)) lies
    in 0 .. rows + 3, the padded column."""
    ov = rows // 2
    vmin, vmax = -2 - ov, rows - ov
    for v0 in range(vmin, vmax + 1):
        assert 0 <= 2 + ov + v0 <= rows + 3


@pytest.mark.parametrize("t", [-300.75, -2.0, -0.5, -1e-6, 0.0, 0.25, 1.0, 255.999, 4e6])
def test_floor_by_magic_number(t):
    """The z-lane kernel's exact floor: for |t| < 2^22, t + 1.5 * 2^23 rounded
    toward -inf is floor(t) + 1.5 * 2^23, and its bits are 0x4B400000 +
    floor(t). Rounding toward -inf is emulated here with numpy's nextafter."""
    t32 = np.float32(t)
    s = np.float32(t32) + np.float32(12582912.0)   # round to nearest
    exact = float(t32) + 12582912.0
    if float(s) > exact:                            # step down to round toward -inf
        s = np.nextafter(s, np.float32(-np.inf))
    assert float(s) - 12582912.0 == np.floor(float(t32))
    bits = int(np.array(s, dtype=np.float32).view(np.uint32))
    assert bits - 0x4B400000 == int(np.floor(float(t32)))
