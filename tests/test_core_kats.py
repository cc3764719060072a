"""Known-answer tests of the host-side time logic that the per-step device tables are built
from (CPU): on/off switches, temporal profiles and apodization windows.

Replays the reference's unit tests on the library's own classes
(tests/unit/core/test_switch.py:29-170, tests/unit/objects/sources/test_profile.py:24-220,
tests/unit/core/test_window.py:22-135), and checks that the parameters the library hands the
kernels (``engine._profile_params``: kind, omega, phase0, ramp, t0, 1 / (2 sigma^2)), fed
through the same formula the device evaluates (a linear ramp clamped to [0, 1] times the
carrier for CW, a Gaussian envelope times the carrier for a pulse), give the reference's
amplitudes, and that the oracle's restatement agrees.
"""

import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import _native as N
from fdtdx_gb300 import engine
from fdtdx_gb300.core import GaussianWindow, OnOffSwitch, TukeyWindow, is_on_at_time_step
from oracle import fdtd_oracle as O


def _sw(**kw):
    base = dict(is_always_off=False, start_time=None, start_after_periods=None, end_time=None, end_after_periods=None,
                on_for_time=None, on_for_periods=None, time_step=0, time_step_duration=1.0, period=None)
    base.update(kw)
    return is_on_at_time_step(**base)


def test_switch_kats():
    assert _sw(is_always_off=True) is False and _sw() is True
    assert _sw(start_time=5.0, time_step=3) is False and _sw(start_time=5.0, time_step=5) is True
    assert _sw(end_time=5.0, time_step=5) is True and _sw(end_time=5.0, time_step=7) is False
    assert _sw(start_after_periods=2.0, period=10.0, time_step=19) is False
    assert _sw(start_after_periods=2.0, period=10.0, time_step=20) is True
    assert _sw(end_after_periods=3.0, period=10.0, time_step=30) is True
    assert _sw(end_after_periods=3.0, period=10.0, time_step=31) is False
    assert _sw(on_for_time=4.0, end_time=10.0, time_step=5) is False and _sw(on_for_time=4.0, end_time=10.0, time_step=6)
    assert _sw(start_time=5.0, on_for_time=3.0, time_step=8) and not _sw(start_time=5.0, on_for_time=3.0, time_step=9)
    assert not _sw(on_for_periods=1.0, end_time=20.0, period=10.0, time_step=9)
    assert _sw(on_for_periods=1.0, end_time=20.0, period=10.0, time_step=10)
    assert _sw(start_time=5.0, on_for_periods=2.0, period=10.0, time_step=25)
    assert not _sw(start_time=5.0, on_for_periods=2.0, period=10.0, time_step=26)
    assert not _sw(start_time=10.0, time_step_duration=0.5, time_step=19)
    assert _sw(start_time=10.0, time_step_duration=0.5, time_step=20)
    with pytest.raises(Exception, match="Need to specify period"):
        _sw(start_after_periods=1.0)
    with pytest.raises(Exception, match="Invalid start time"):
        _sw(start_time=0.0, start_after_periods=1.0, period=10.0)
    with pytest.raises(Exception, match="Invalid end time"):
        _sw(end_time=10.0, end_after_periods=2.0, period=5.0)


def test_switch_lists():
    assert OnOffSwitch().calculate_on_list(5, 1.0) == [True] * 5
    assert OnOffSwitch().is_default_always_on
    for kw in ({"interval": 2}, {"start_time": 0.0}, {"end_time": 1.0}, {"fixed_on_time_steps": [0]},
               {"is_always_off": True}):
        assert not OnOffSwitch(**kw).is_default_always_on
    assert OnOffSwitch(interval=3).calculate_on_list(7, 1.0) == [True, False, False, True, False, False, True]
    assert OnOffSwitch(fixed_on_time_steps=[1, 3, 4]).calculate_on_list(6, 1.0) == [False, True, False, True, True,
                                                                                     False]
    assert OnOffSwitch(start_time=1.0, end_time=3.0).calculate_time_step_to_on_arr_idx(6, 1.0) == [-1, 0, 1, 2, -1, -1]


def _device_amp(profile, wave, dt: float, tau_steps):
    """The device's profile evaluation on the library's table parameters."""
    kind, omega, phase0, ramp_inv, t0s, inv2s2 = engine._profile_params(profile, wave, dt)
    tau = np.asarray(tau_steps, dtype=np.float64)
    carrier = np.cos(omega * dt * tau + phase0)
    if kind == N.PROFILE_CW:
        return np.clip(tau * ramp_inv, 0.0, 1.0) * carrier
    return np.exp(-((tau - t0s) ** 2) * inv2s2) * carrier


def test_single_frequency_profile_kats():
    p = fx.SingleFrequencyProfile()
    assert p.phase_shift == math.pi and p.num_startup_periods == 4
    T = 1e-12
    p0 = fx.SingleFrequencyProfile(phase_shift=0.0, num_startup_periods=4)
    assert abs(p0.get_amplitude(0.0, T)) < 1e-12
    assert abs(p0.get_amplitude(4 * T, T) - 1.0) < 1e-6 and abs(p0.get_amplitude(2 * T, T) - 0.5) < 1e-6
    p1 = fx.SingleFrequencyProfile(phase_shift=math.pi, num_startup_periods=1)
    assert abs(p1.get_amplitude(2 * T, T) + 1.0) < 1e-6
    q = fx.SingleFrequencyProfile(phase_shift=0.0, num_startup_periods=1)
    assert abs(q.get_amplitude(2 * T, T, phase_shift=math.pi / 2)) < 1e-6
    got = [q.get_amplitude(10 * T + f * T, T) for f in (0.0, 0.25, 0.5, 0.75, 1.0)]
    assert np.allclose(got, [1.0, 0.0, -1.0, 0.0, 1.0], atol=1e-6)
    # the device's evaluation on the library's parameters, and the oracle, against get_amplitude
    dt = T / 37.3
    wave = fx.WaveCharacter(wavelength=T * 299792458.0, phase_shift=0.3)
    for prof in (fx.SingleFrequencyProfile(), fx.SingleFrequencyProfile(phase_shift=0.0, num_startup_periods=2)):
        tau = np.linspace(-3.0, 400.0, 1213)
        want = np.array([prof.get_amplitude(t * dt, wave.get_period(), wave.phase_shift) for t in tau])
        assert np.allclose(_device_amp(prof, wave, dt, tau), want, atol=1e-9)
        orc = O.profile_amplitude(prof, torch.tensor(tau * dt, dtype=torch.float64), wave.get_period(),
                                  wave.phase_shift).numpy()
        assert np.allclose(orc, want, atol=1e-9)


def test_gaussian_pulse_profile_kats():
    center, width = fx.WaveCharacter(wavelength=1e-6), fx.WaveCharacter(wavelength=2e-6)
    prof = fx.GaussianPulseProfile(center_wave=center, spectral_width=width)
    t = np.linspace(0, 5e-14, 60)
    sigma_t = 1.0 / (2 * np.pi * width.get_frequency())
    env = np.exp(-((t - 6 * sigma_t) ** 2) / (2 * sigma_t**2))
    carrier = np.real(np.exp(-1j * (2 * np.pi * center.get_frequency() * t + center.phase_shift)))
    got = np.array([prof.get_amplitude(x, 1e-15) for x in t])
    assert np.allclose(got, env * carrier, rtol=1e-4, atol=1e-5)
    wide = fx.GaussianPulseProfile(spectral_width=fx.WaveCharacter(frequency=1e13),
                                   center_wave=fx.WaveCharacter(frequency=193.4e12))
    period = 1 / 193.4e12
    t_peak = 6 * wide.sigma_t
    assert abs(wide.get_amplitude(t_peak, period)) > abs(wide.get_amplitude(t_peak - 5e-13, period))
    dt = 1e-17
    for pr, wave in ((prof, fx.WaveCharacter(wavelength=1e-6, phase_shift=0.7)), (wide, center)):
        tau = np.linspace(0.0, 12 * pr.sigma_t / dt, 997)
        want = np.array([pr.get_amplitude(x * dt, wave.get_period(), wave.phase_shift) for x in tau])
        assert np.allclose(_device_amp(pr, wave, dt, tau), want, atol=1e-9)
        orc = O.profile_amplitude(pr, torch.tensor(tau * dt, dtype=torch.float64), wave.get_period(),
                                  wave.phase_shift).numpy()
        assert np.allclose(orc, want, atol=1e-9)


def test_window_kats():
    t = np.linspace(0, 1e-12, 50)
    g = GaussianWindow(center_time=5e-13, sigma_time=1e-13).get_window(t)
    assert np.allclose(g, np.exp(-((t - 5e-13) ** 2) / (2 * 1e-26)), atol=1e-7)
    x = np.linspace(0, 1, 101)
    w = TukeyWindow(start_time=0.0, end_time=1.0, alpha=0.5).get_window(x)
    assert abs(w[0]) < 1e-6 and abs(w[-1]) < 1e-6 and abs(w[50] - 1.0) < 1e-6
    assert np.allclose(TukeyWindow(start_time=0.0, end_time=1.0, alpha=0.0).get_window(np.linspace(0, 1, 51)), 1.0)
    hann = TukeyWindow(start_time=0.0, end_time=1.0, alpha=1.0).get_window(np.linspace(0, 1, 51))
    assert np.allclose(hann, 0.5 * (1 - np.cos(2 * np.pi * np.linspace(0, 1, 51))), atol=1e-6)
    out = TukeyWindow(start_time=0.0, end_time=1.0, alpha=0.5).get_window(np.array([-0.1, 0.5, 1.1]))
    assert out[0] == 0.0 and out[2] == 0.0
    tt = np.linspace(-1e-12, 2e-12, 200)
    assert (GaussianWindow(center_time=5e-13, sigma_time=1e-13).get_window(tt) >= 0).all()
    assert (TukeyWindow(start_time=0.0, end_time=1e-12, alpha=0.5).get_window(tt) >= 0).all()
    for sigma in (0.0, -1e-13):
        with pytest.raises(ValueError, match="sigma_time must be positive"):
            GaussianWindow(center_time=5e-13, sigma_time=sigma)
    for end in (0.0, -1e-12, 1e-12):
        with pytest.raises(ValueError, match="end_time must exceed start_time"):
            TukeyWindow(start_time=1e-12, end_time=end)
    for alpha in (-0.1, 1.5):
        with pytest.raises(ValueError, match=r"alpha must lie in \[0, 1\]"):
            TukeyWindow(start_time=0.0, end_time=1e-12, alpha=alpha)
