"""ts.host_buffer: page-locked huge-page host tensors for transfers."""
import gc

import numpy as np
import pytest
import torch

import tomosipo_gb300 as ts
from tomosipo_gb300 import hostmem


def test_huge_page_size_is_a_power_of_two():
    hp = hostmem.huge_page_bytes()
    assert hp >= 4096 and hp & (hp - 1) == 0


@pytest.mark.parametrize("shape", [(3, 4, 5), 7, (0, 3)])
def test_host_buffer_shape_dtype_and_writable(shape):
    t = ts.host_buffer(shape, dtype=torch.float32)
    assert t.dtype == torch.float32 and t.device.type == "cpu"
    assert tuple(t.shape) == (shape if isinstance(shape, tuple) else (shape,))
    t.fill_(2.5)
    assert bool(torch.all(t == 2.5))


def test_host_buffer_other_dtypes():
    for dt in (torch.float64, torch.int32, torch.bool):
        t = ts.host_buffer((4, 2), dtype=dt)
        assert t.dtype == dt and tuple(t.shape) == (4, 2)


def _rss_bytes():
    with open("/proc/self/status") as f:
        for line in f:
            if line.startswith("VmRSS:"):
                return int(line.split()[1]) * 1024
    return 0


@pytest.mark.gpu
def test_host_buffer_is_pinned_projects_and_is_released(native_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda", 0)
    vg = ts.volume(shape=32, size=1)
    pg = ts.cone(angles=48, shape=(32, 48), size=np.sqrt(2), cone_angle=0.5)
    A = ts.operator(vg, pg)
    x = torch.rand(A.domain_shape, generator=torch.Generator().manual_seed(0))
    xh = ts.host_buffer(A.domain_shape)
    yh = ts.host_buffer(A.range_shape)
    assert xh.is_pinned() and yh.is_pinned()
    xh.copy_(x)
    A(xh, out=yh)
    assert torch.equal(yh, A(x.to(dev)).cpu())
    # views keep the mapping; freeing the last one releases it
    v = xh[3:5]
    del xh
    gc.collect()
    assert torch.equal(v, x[3:5])
    del v, yh
    gc.collect()
    before = _rss_bytes()
    for _ in range(8):
        t = ts.host_buffer((64 << 20,))  # 256 MiB, touched by registration
        t[::4096].fill_(1.0)
        del t
        gc.collect()
    assert _rss_bytes() - before < (256 << 20), "host buffers are not released"
