"""The phasor detector's per-step device tables against the reference's DFT-subsampling and
apodization tests (CPU).

The kernels accumulate ``state += w[t] * value(t)`` on every step whose slot is set, with the
complex weight w[t] = exp(i omega t dt) * scale * window[t] that ``engine.detector_tables``
builds on the host.  Driving that accumulation with the reference's synthetic signals replays
tests/unit/objects/detectors/test_phasor_subsample.py:29-180 and
tests/unit/objects/detectors/test_apodization.py:37-200 on the tables the GPU reads.
"""

import math

import numpy as np
import pytest

import fdtdx_gb300 as fx
from fdtdx_gb300 import engine
from fdtdx_gb300.core import GaussianWindow, TukeyWindow


def _cfg(time, spacing):
    return fx.SimulationConfig(time=time, grid=fx.UniformGrid(spacing))


def _tables(det, cfg):
    det.place_on_grid(((0, 4), (0, 4), (0, 1)))
    slot, w = engine.detector_tables(det, cfg)
    return slot[1:-1], (w[1:-1, :, 0] + 1j * w[1:-1, :, 1]).astype(np.complex128)  # steps 0 .. T-1


def _accumulate(det, cfg, signal):
    slot, w = _tables(det, cfg)
    T = cfg.time_steps_total
    return sum(w[t, 0] * signal(t) for t in range(T) if slot[t] >= 0)


def test_default_and_explicit_stride():
    cfg = _cfg(1e-13, 1e-7)
    wc = fx.WaveCharacter(frequency=1e14)
    T = cfg.time_steps_total
    slot1, _ = _tables(fx.PhasorDetector(name="a", wave_characters=(wc,)), cfg)
    assert (slot1 >= 0).all()
    slot3, _ = _tables(fx.PhasorDetector(name="b", wave_characters=(wc,), dft_subsample=3), cfg)
    assert np.array_equal(np.nonzero(slot3 >= 0)[0], np.arange(T)[::3])
    auto = fx.PhasorDetector(name="c", wave_characters=(wc,), dft_subsample="auto")
    want = max(1, math.floor(1.0 / (12 * 1e14 * cfg.time_step_duration)))
    assert want > 1 and auto.resolve_dft_stride(cfg) == want


def test_pulse_and_continuous_scaling_with_stride():
    cfg = _cfg(1e-13, 1e-7)
    wc = fx.WaveCharacter(frequency=1e14)
    _, w1 = _tables(fx.PhasorDetector(name="a", wave_characters=(wc,), scaling_mode="pulse"), cfg)
    _, w3 = _tables(fx.PhasorDetector(name="b", wave_characters=(wc,), scaling_mode="pulse", dft_subsample=3), cfg)
    assert abs(w3[0, 0] - 3.0 * w1[0, 0]) < 1e-6 * abs(w1[0, 0])
    slot4, w4 = _tables(fx.PhasorDetector(name="c", wave_characters=(wc,), dft_subsample=4), cfg)
    assert abs(w4[0, 0] - 2.0 / int((slot4 >= 0).sum())) < 1e-7


def test_subsampled_phasor_recovers_cw_amplitude():
    cfg = _cfg(1e-13, 1e-7)
    f = 1e14
    om, dt = 2 * math.pi * f, cfg.time_step_duration
    wc = fx.WaveCharacter(frequency=f)
    exact = abs(_accumulate(fx.PhasorDetector(name="a", wave_characters=(wc,)), cfg, lambda t: math.cos(om * t * dt)))
    auto_det = fx.PhasorDetector(name="b", wave_characters=(wc,), dft_subsample="auto")
    assert auto_det.resolve_dft_stride(cfg) > 1
    auto = abs(_accumulate(auto_det, cfg, lambda t: math.cos(om * t * dt)))
    assert exact == pytest.approx(1.0, abs=0.05) and auto == pytest.approx(exact, rel=0.05)


def test_apodization_tables():
    cfg = _cfg(2e-13, 1e-7)
    T, dt = cfg.time_steps_total, cfg.time_step_duration
    wc = fx.WaveCharacter(wavelength=1e-6)
    om = 2 * math.pi * wc.get_frequency()

    def cw(t):
        return math.cos(om * t * dt)

    plain = fx.PhasorDetector(name="p", wave_characters=(wc,), reduce_volume=True)
    assert abs(_accumulate(plain, cfg, cw)) == pytest.approx(1.0, abs=2e-3)
    end = (T - 1) * dt
    for stride in (1, 2, 3, 4):
        tuk = fx.PhasorDetector(name="t", wave_characters=(wc,), reduce_volume=True, dft_subsample=stride,
                                apodization=TukeyWindow(start_time=0.0, end_time=end, alpha=0.5))
        assert abs(_accumulate(tuk, cfg, cw)) == pytest.approx(1.0, abs=1e-5)
    # an alpha = 0 Tukey over the whole recording is the rectangular window, bit for bit
    rect = fx.PhasorDetector(name="r", wave_characters=(wc,), reduce_volume=True,
                             apodization=TukeyWindow(start_time=0.0, end_time=end, alpha=0.0))
    assert np.array_equal(_tables(rect, cfg)[1], _tables(plain, cfg)[1])
    # a window changes a transient's spectrum

    def decay(t):
        return math.exp(-3.0 * t / T) * math.cos(om * t * dt)

    r = _accumulate(fx.PhasorDetector(name="a", wave_characters=(wc,), reduce_volume=True, scaling_mode="pulse"),
                    cfg, decay)
    a = _accumulate(fx.PhasorDetector(name="b", wave_characters=(wc,), reduce_volume=True, scaling_mode="pulse",
                                      apodization=TukeyWindow(start_time=0.0, end_time=end, alpha=0.8)), cfg, decay)
    assert abs(r - a) > 1e-3 * abs(r)
    # windows whose gain over the recording is zero are refused
    for win in (TukeyWindow(start_time=10 * end, end_time=11 * end),
                GaussianWindow(center_time=1e6 * end, sigma_time=1e-18)):
        with pytest.raises(Exception, match="must be finite and positive"):
            _tables(fx.PhasorDetector(name="z", wave_characters=(wc,), apodization=win), cfg)
    with pytest.raises(Exception, match="must be a TemporalWindow"):
        fx.PhasorDetector(name="s", wave_characters=(wc,), apodization=fx.SingleFrequencyProfile())
