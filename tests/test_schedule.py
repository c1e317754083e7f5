"""The forward projector's tile order (tsgb_tuning), restated on the host.

``fp_schedule_tile`` in ``tomosipo_gb300/csrc/device_common.cuh`` maps a
linear block index to (row block, column block, angle pair): groups of angle
pairs, inside a group the detector patches strip by strip, inside a patch the
pairs and then the tiles with row blocks fastest. This restatement must be a
bijection onto all tiles for ragged sizes; the GPU tests check that every
schedule gives bit-identical sinograms.
"""
import itertools

import numpy as np
import pytest


def tile(b, rows, cols, pairs, pr_, pc_, gp):
    pr_, pc_, gp = min(pr_, rows), min(pc_, cols), min(gp, pairs)
    per_pair = rows * cols
    full_group = per_pair * gp
    grp, b = divmod(b, full_group)
    gsz = min(gp, pairs - grp * gp)
    full_strip = gsz * pr_ * cols
    pr, b = divmod(b, full_strip)
    rsz = min(pr_, rows - pr * pr_)
    full_patch = gsz * rsz * pc_
    pc, b = divmod(b, full_patch)
    csz = min(pc_, cols - pc * pc_)
    q, t = divmod(b, rsz * csz)
    return pr * pr_ + t % rsz, pc * pc_ + t // rsz, grp * gp + q


@pytest.mark.parametrize("rows,cols,pairs", [(1, 1, 1), (3, 5, 7), (16, 96, 4), (5, 13, 9)])
@pytest.mark.parametrize("pr_,pc_,gp", [(1, 1, 1), (2, 3, 2), (4, 16, 8), (7, 64, 100)])
def test_tile_order_is_a_bijection(rows, cols, pairs, pr_, pc_, gp):
    n = rows * cols * pairs
    seen = [tile(b, rows, cols, pairs, pr_, pc_, gp) for b in range(n)]
    assert sorted(seen) == sorted(itertools.product(range(rows), range(cols), range(pairs)))


def test_patch_tiles_are_contiguous():
    # first group, first patch: its pairs x tiles come first, row blocks fastest
    seen = [tile(b, 8, 32, 16, 4, 16, 8) for b in range(4 * 16 * 8)]
    assert {s[0] for s in seen} == set(range(4))
    assert {s[1] for s in seen} == set(range(16))
    assert {s[2] for s in seen} == set(range(8))
    assert seen[:3] == [(0, 0, 0), (1, 0, 0), (2, 0, 0)]


@pytest.mark.parametrize("nang", [16, 17, 40, 100, 360, 1024, 4097])
def test_pipeline_chunk_bounds(nang):
    """Angle chunks of a streamed projection cover every angle once, in order;
    the chunk whose transfer is exposed (the backprojection's first, the
    forward projection's last) is the smallest, and the rest grow by at most
    the direction's growth factor from it, the farthest also taking a
    remainder smaller than one more step."""
    from tomosipo_gb300.projector import PIPELINE_GROWTH_BP, PIPELINE_GROWTH_FP, _chunk_bounds

    for forward, growth in ((False, PIPELINE_GROWTH_BP), (True, PIPELINE_GROWTH_FP)):
        b = [int(v) for v in _chunk_bounds(nang, forward)]
        sizes = np.diff(b)
        assert b[0] == 0 and b[-1] == nang and np.all(sizes >= 1)
        grow = sizes if not forward else sizes[::-1]
        assert grow[0] == min(sizes) <= max(1, nang // 32)
        assert np.all(grow[1:-1] <= grow[:-2] * growth)
        if len(grow) > 1:
            assert grow[-1] < grow[-2] * growth * (growth + 1)
    assert list(_chunk_bounds(1024, False)) == [0, 32, 288, 1024]
    assert list(_chunk_bounds(1024, True)) == [0, 544, 800, 928, 992, 1024]
