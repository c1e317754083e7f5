"""FDK's host stages (``tomosipo_gb300.fdk``: cosine weights, the FFT ramp
filter and the per-angle weights) against the FP64 NumPy FDK oracle's direct
convolution, on CPU tensors (the GPU tests cover the backprojection)."""
import numpy as np
import pytest
import torch

import tomosipo_gb300 as ts
from oracle import fdk_oracle
from tests.helpers import helical_cone_vec, rel_l2
from tomosipo_gb300 import fdk


# a scan of pi + 0.5 rad: the detector's fan half-angle is about 0.17 rad
SHORT = np.linspace(0, np.pi + 0.5, 17, endpoint=False)


def _scans():
    kw = dict(shape=(9, 13), size=(1.2, 1.6), src_orig_dist=3, src_det_dist=4.5)
    circular = ts.cone(angles=17, **kw)
    lift = np.stack([np.linspace(-0.2, 0.2, 17), np.zeros(17), np.zeros(17)], axis=1)
    rot = ts.rotate(pos=0, axis=(1.0, 0.4, -0.3), angles=0.5)
    # per-angle source and detector jitter: the cosine weights differ per angle
    # (the other scans share one weight map)
    jittered = helical_cone_vec(17, (9, 13), (1.2, 1.6), 3.0, 1.5, pitch=0.0, jitter=0.5,
                                voxel=0.05)
    return {"circular": circular, "helical": ts.translate(lift) * circular.to_vec(),
            "rotated": rot * circular.to_vec(), "short": ts.cone(angles=SHORT, **kw),
            "short_rotated_reversed": rot * ts.cone(angles=-SHORT, **kw).to_vec(),
            "jittered": jittered}


@pytest.mark.parametrize("scan", ["circular", "helical", "rotated", "short",
                                  "short_rotated_reversed", "jittered"])
def test_filter_and_angle_weights_match_the_oracle(scan):
    pg = _scans()[scan]
    short = scan.startswith("short")
    vg = ts.volume(shape=(10, 12, 14), size=(0.8, 1, 1.1), pos=(0.05, -0.1, 0.02))
    y = np.random.default_rng(1).random((9, 17, 13)).astype(np.float32)
    q = fdk.fdk_filter(vg, pg, torch.from_numpy(y), short_scan=short).double().numpy()
    ref = fdk_oracle.filtered(vg, pg, y.astype(np.float64), short_scan=short)
    assert rel_l2(q, ref) < 1e-5  # measured 1.2e-7
    assert np.abs(fdk.fdk_constants(vg, pg)[2] - fdk_oracle.angle_weights(vg, pg)).max() < 1e-12
    if short:
        assert np.abs(fdk.short_scan_weights(vg, pg) - fdk_oracle.parker(vg, pg)).max() < 1e-12


def test_rotation_axis_of_a_rotated_scan_is_the_rotated_z_axis():
    rot = ts.rotate(pos=0, axis=(1.0, 0.4, -0.3), angles=0.5)
    pg = _scans()["rotated"]
    V = np.asarray(pg.det_v, dtype=np.float64)
    axis, e1, e2 = fdk.rotation_frame(V)
    z = np.asarray(rot.transform_vec(np.array([[1.0, 0, 0]])), dtype=np.float64).reshape(3)
    assert abs(abs(axis @ (z / np.linalg.norm(z))) - 1) < 1e-12
    assert abs(e1 @ axis) < 1e-12 and abs(e2 @ axis) < 1e-12 and abs(e1 @ e2) < 1e-12
    # full-circle angle steps about the rotated axis through the origin (the
    # anchor of an odd-sided volume centred there) are 2 pi / 17, as about z
    w = fdk.fdk_constants(ts.volume(shape=9, size=1), pg)[2]
    assert np.abs(w - np.pi / 17).max() < 1e-12


def test_parker_weights_of_each_redundant_pair_sum_to_one():
    delta = 0.3
    rng = np.random.default_rng(2)
    gamma = rng.uniform(-delta, delta, 200)
    beta = rng.uniform(0, np.pi + 2 * delta, 200)
    conj = beta + np.pi + 2 * gamma  # the same line, measured later ...
    early = conj <= np.pi + 2 * delta
    beta_e, gamma_e = beta[early], gamma[early]
    s = fdk.parker_weights(beta_e, gamma_e, delta) + fdk.parker_weights(
        beta_e + np.pi + 2 * gamma_e, -gamma_e, delta)
    assert np.abs(s - 1).max() < 1e-12
    # ... and lines measured once have weight 1
    once = (beta >= 2 * (delta - gamma)) & (beta <= np.pi - 2 * gamma)
    assert np.all(fdk.parker_weights(beta[once], gamma[once], delta) == 1)
    assert np.all(fdk.parker_weights(np.array([-0.1, np.pi + 2 * delta + 0.1]), 0.0, delta) == 0)


def test_short_scan_needs_pi_plus_the_fan_angle():
    pg = ts.cone(angles=np.linspace(0, np.pi + 0.2, 17, endpoint=False), shape=(9, 13),
                 size=(1.2, 1.6), src_orig_dist=3, src_det_dist=4.5)
    with pytest.raises(ValueError, match="pi plus the fan angle"):
        fdk.short_scan_weights(ts.volume(shape=8), pg)


def test_ramp_spectrum_is_the_zero_padded_ram_lak_kernel():
    """The spectrum of the Ram-Lak kernel truncated to |n| < cols: its DC term
    is the kernel's sum, 1/4 - 2 sum_{odd n < cols} 1/(pi n)^2 (small and
    positive), and it rises to about |f| = 1/2 at the Nyquist frequency."""
    spec, length = fdk.ramp_spectrum(13, "cpu")
    assert length == fdk.fft_length(13) == 28 and spec.shape == (15,)
    odd = np.arange(1, 13, 2)
    assert spec[0].item() == pytest.approx(0.25 - 2 * np.sum(1 / (np.pi * odd) ** 2), abs=1e-6)
    assert torch.all(spec[1:] > spec[:-1]) and spec[-1].item() == pytest.approx(0.5, abs=0.01)


@pytest.mark.parametrize("cols", [1, 9, 13, 192, 384, 768, 1000, 1021])
def test_fft_length_avoids_wrap_around_with_fast_radices(cols):
    """The filter's FFT length holds a linear convolution of a row with the
    kernel's 2 cols - 1 taps, is even, and has only the prime factors 2, 3, 5
    and 7; it is the smallest such length."""
    n = fdk.fft_length(cols)

    def smooth(m):
        for f in (2, 3, 5, 7):
            while m % f == 0:
                m //= f
        return m == 1

    assert n >= 2 * cols - 1 and n % 2 == 0 and smooth(n)
    assert not any(smooth(m) and m % 2 == 0 for m in range(max(2 * cols - 1, 2), n))


def test_fdk_rejects_parallel_beams():
    with pytest.raises(ValueError):
        fdk.fdk_constants(ts.volume(shape=4), ts.parallel(angles=3, shape=4))


@pytest.mark.parametrize("scan", ["circular", "jittered"])
def test_filter_does_not_depend_on_the_angle_chunk(scan):
    """The filter runs its angles in chunks (as many as fit its buffer budget);
    every angle's arithmetic is the same whatever the chunk, so chunks of 1, 5
    and all 17 angles give equal results."""
    pg = _scans()[scan]
    vg = ts.volume(shape=(10, 12, 14), size=(0.8, 1, 1.1), pos=(0.05, -0.1, 0.02))
    y = torch.from_numpy(np.random.default_rng(2).random((9, 17, 13)).astype(np.float32))
    ref = fdk.fdk_filter(vg, pg, y, angle_chunk=17)
    for chunk in (1, 5, None):
        assert torch.equal(fdk.fdk_filter(vg, pg, y, angle_chunk=chunk), ref), chunk
    for bad in (0, -3):
        with pytest.raises(ValueError, match="angle_chunk"):
            fdk.fdk_filter(vg, pg, y, angle_chunk=bad)
