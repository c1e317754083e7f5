"""FDK's host stages (``tomosipo_gb300.fdk``: cosine weights, the FFT ramp
filter and the per-angle weights) against the FP64 NumPy FDK oracle's direct
convolution, on CPU tensors (the GPU tests cover the backprojection)."""
import numpy as np
import pytest
import torch

import tomosipo_gb300 as ts
from oracle import fdk_oracle
from tests.helpers import rel_l2
from tomosipo_gb300 import fdk


def _scans():
    circular = ts.cone(angles=17, shape=(9, 13), size=(1.2, 1.6), src_orig_dist=3,
                       src_det_dist=4.5)
    lift = np.stack([np.linspace(-0.2, 0.2, 17), np.zeros(17), np.zeros(17)], axis=1)
    return {"circular": circular, "helical": ts.translate(lift) * circular.to_vec()}


@pytest.mark.parametrize("scan", ["circular", "helical"])
def test_filter_and_angle_weights_match_the_oracle(scan):
    pg = _scans()[scan]
    vg = ts.volume(shape=(10, 12, 14), size=(0.8, 1, 1.1), pos=(0.05, -0.1, 0.02))
    y = np.random.default_rng(1).random((9, 17, 13)).astype(np.float32)
    q = fdk.fdk_filter(vg, pg, torch.from_numpy(y)).double().numpy()
    assert rel_l2(q, fdk_oracle.filtered(vg, pg, y.astype(np.float64))) < 1e-5  # measured 1.2e-7
    assert np.abs(fdk.fdk_constants(vg, pg)[2] - fdk_oracle.angle_weights(vg, pg)).max() < 1e-12


def test_ramp_spectrum_is_the_zero_padded_ram_lak_kernel():
    """The spectrum of the Ram-Lak kernel truncated to |n| < cols: its DC term
    is the kernel's sum, 1/4 - 2 sum_{odd n < cols} 1/(pi n)^2 (small and
    positive), and it rises to about |f| = 1/2 at the Nyquist frequency."""
    spec, length = fdk.ramp_spectrum(13, "cpu")
    assert length == 32 and spec.shape == (17,)
    odd = np.arange(1, 13, 2)
    assert spec[0].item() == pytest.approx(0.25 - 2 * np.sum(1 / (np.pi * odd) ** 2), abs=1e-6)
    assert torch.all(spec[1:] > spec[:-1]) and spec[-1].item() == pytest.approx(0.5, abs=0.01)


def test_fdk_rejects_parallel_beams():
    with pytest.raises(ValueError):
        fdk.fdk_constants(ts.volume(shape=4), ts.parallel(angles=3, shape=4))
