"""Wave characters, on/off switches, temporal source profiles and detector windows.

Host-side value objects with the field names and semantics of fdtdx:

* ``WaveCharacter``        fdtdx/core/wavelength.py:5-65
* ``OnOffSwitch``          fdtdx/core/switch.py:6-209
* ``SingleFrequencyProfile`` / ``GaussianPulseProfile``  fdtdx/objects/sources/profile.py:253-345
* ``GaussianWindow`` / ``TukeyWindow``  fdtdx/core/window.py:16-120

The profiles evaluate in float64 numpy on the host.  The device kernels never
call these: the host turns them into per-step phase/envelope parameters (see
``fdtdx_gb300.engine``) and the kernels evaluate the carrier with a reduced
phase argument.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from fdtdx_gb300 import constants


@dataclass(frozen=True)
class WaveCharacter:
    """A free-space wave given by exactly one of period, wavelength or frequency."""

    phase_shift: float = 0.0
    period: float | None = None
    wavelength: float | None = None
    frequency: float | None = None

    def __post_init__(self):
        if sum(x is not None for x in (self.period, self.wavelength, self.frequency)) != 1:
            raise Exception("Need to set exactly one of Period, Frequency or Wavelength in WaveCharacter")

    def get_period(self) -> float:
        if self.period is not None:
            return self.period
        if self.wavelength is not None:
            return self.wavelength / constants.c
        return 1.0 / self.frequency  # type: ignore[operator]

    def get_wavelength(self) -> float:
        if self.wavelength is not None:
            return self.wavelength
        if self.period is not None:
            return self.period * constants.c
        return constants.c / self.frequency  # type: ignore[operator]

    def get_frequency(self) -> float:
        if self.frequency is not None:
            return self.frequency
        if self.period is not None:
            return 1.0 / self.period
        return constants.c / self.wavelength  # type: ignore[operator]


def is_on_at_time_step(
    is_always_off: bool,
    start_time: float | None,
    start_after_periods: float | None,
    end_time: float | None,
    end_after_periods: float | None,
    on_for_time: float | None,
    on_for_periods: float | None,
    time_step: int,
    time_step_duration: float,
    period: float | None,
) -> bool:
    """Whether a switch is on at ``time_step`` (fdtdx/core/switch.py:112-209)."""
    if is_always_off:
        return False
    need_period = any(x is not None for x in (start_after_periods, end_after_periods, on_for_periods))
    if need_period and period is None:
        raise Exception("Need to specify period!")
    n_start = sum(
        [
            start_time is not None,
            start_after_periods is not None,
            on_for_time is not None and end_time is not None,
            on_for_periods is not None and end_time is not None,
            on_for_time is not None and end_after_periods is not None,
            on_for_periods is not None and end_after_periods is not None,
        ]
    )
    if n_start > 1:
        raise Exception("Invalid start time specification!")
    if n_start == 0:
        start_time = 0
    n_end = sum(
        [
            end_time is not None,
            end_after_periods is not None,
            on_for_time is not None and start_time is not None,
            on_for_periods is not None and start_time is not None,
            on_for_time is not None and start_after_periods is not None,
            on_for_periods is not None and start_after_periods is not None,
        ]
    )
    if n_end > 1:
        raise Exception("Invalid end time specification!")
    if n_end == 0:
        end_time = math.inf
    if start_after_periods is not None:
        start_time = start_after_periods * period  # type: ignore[operator]
    if end_after_periods is not None:
        end_time = end_after_periods * period  # type: ignore[operator]
    if on_for_periods is not None:
        on_for_time = on_for_periods * period  # type: ignore[operator]
    if start_time is None and on_for_time is not None:
        start_time = end_time - on_for_time  # type: ignore[operator]
    if end_time is None and on_for_time is not None:
        end_time = start_time + on_for_time  # type: ignore[operator]
    t = time_step * time_step_duration
    return bool(start_time <= t <= end_time)  # type: ignore[operator]


@dataclass(frozen=True)
class OnOffSwitch:
    """Per-time-step on/off schedule of a source or detector."""

    start_time: float | None = None
    start_after_periods: float | None = None
    end_time: float | None = None
    end_after_periods: float | None = None
    on_for_time: float | None = None
    on_for_periods: float | None = None
    period: float | None = None
    fixed_on_time_steps: Sequence[int] | None = None
    is_always_off: bool = False
    interval: int = 1

    @property
    def is_default_always_on(self) -> bool:
        return (
            not self.is_always_off
            and self.fixed_on_time_steps is None
            and self.interval == 1
            and self.start_time is None
            and self.start_after_periods is None
            and self.end_time is None
            and self.end_after_periods is None
            and self.on_for_time is None
            and self.on_for_periods is None
            and self.period is None
        )

    def calculate_on_list(self, num_total_time_steps: int, time_step_duration: float) -> list[bool]:
        if self.fixed_on_time_steps is not None:
            on = [False] * num_total_time_steps
            for t in self.fixed_on_time_steps:
                on[t] = True
            return on
        out = []
        for t in range(num_total_time_steps):
            cur = is_on_at_time_step(
                self.is_always_off,
                self.start_time,
                self.start_after_periods,
                self.end_time,
                self.end_after_periods,
                self.on_for_time,
                self.on_for_periods,
                t,
                time_step_duration,
                self.period,
            )
            out.append(cur and t % self.interval == 0)
        return out

    def calculate_time_step_to_on_arr_idx(self, num_total_time_steps: int, time_step_duration: float) -> list[int]:
        on = self.calculate_on_list(num_total_time_steps, time_step_duration)
        idx, counter = [-1] * num_total_time_steps, 0
        for t in range(num_total_time_steps):
            if on[t]:
                idx[t] = counter
                counter += 1
        return idx


class TemporalProfile:
    """Base class of the source time signals."""

    def get_amplitude(self, time, period: float, phase_shift: float = 0.0):
        raise NotImplementedError


@dataclass(frozen=True)
class SingleFrequencyProfile(TemporalProfile):
    """cos(2 pi t / T + phase) with a linear start-up ramp over ``num_startup_periods`` periods."""

    phase_shift: float = math.pi
    num_startup_periods: int = 4

    def get_amplitude(self, time, period: float, phase_shift: float = 0.0):
        time = np.asarray(time, dtype=np.float64)
        phase = 2 * math.pi * time / period + phase_shift + self.phase_shift
        ramp = np.clip(time / (self.num_startup_periods * period), 0.0, 1.0)
        return ramp * np.cos(phase)


@dataclass(frozen=True)
class GaussianPulseProfile(TemporalProfile):
    """Gaussian envelope exp(-(t - 6 sigma)^2 / 2 sigma^2) times the carrier, sigma = 1 / (2 pi df)."""

    spectral_width: WaveCharacter = field(default_factory=lambda: WaveCharacter(frequency=1.0))
    center_wave: WaveCharacter = field(default_factory=lambda: WaveCharacter(frequency=1.0))

    def __post_init__(self):
        if self.spectral_width.phase_shift != 0.0:
            raise ValueError(
                "spectral_width should not have a phase_shift. Phase shifts should only be applied to center_wave."
            )

    @property
    def sigma_t(self) -> float:
        return 1.0 / (2 * math.pi * self.spectral_width.get_frequency())

    def get_amplitude(self, time, period: float, phase_shift: float = 0.0):
        del period
        time = np.asarray(time, dtype=np.float64)
        sigma_t = self.sigma_t
        t0 = 6 * sigma_t
        env = np.exp(-((time - t0) ** 2) / (2.0 * sigma_t**2))
        carrier = np.cos(
            2 * math.pi * self.center_wave.get_frequency() * time + phase_shift + self.center_wave.phase_shift
        )
        return env * carrier


class TemporalWindow:
    """Carrier-free apodization window of a phasor detector."""

    def get_window(self, time):
        raise NotImplementedError


@dataclass(frozen=True)
class GaussianWindow(TemporalWindow):
    center_time: float = 0.0
    sigma_time: float = 1.0

    def __post_init__(self):
        if not self.sigma_time > 0:
            raise ValueError(f"sigma_time must be positive, got {self.sigma_time}")

    def get_window(self, time):
        time = np.asarray(time, dtype=np.float64)
        return np.exp(-((time - self.center_time) ** 2) / (2.0 * self.sigma_time**2))


@dataclass(frozen=True)
class TukeyWindow(TemporalWindow):
    start_time: float = 0.0
    end_time: float = 1.0
    alpha: float = 0.5

    def __post_init__(self):
        if not self.end_time > self.start_time:
            raise ValueError(f"end_time must exceed start_time, got {self.start_time} and {self.end_time}")
        if not 0.0 <= self.alpha <= 1.0:
            raise ValueError(f"alpha must lie in [0, 1], got {self.alpha}")

    def get_window(self, time):
        time = np.asarray(time, dtype=np.float64)
        x = (time - self.start_time) / (self.end_time - self.start_time)
        inside = (x >= 0.0) & (x <= 1.0)
        if self.alpha <= 0.0:
            return np.where(inside, 1.0, 0.0)
        half = self.alpha / 2.0
        left = 0.5 * (1.0 + np.cos(np.pi * (x / half - 1.0)))
        right = 0.5 * (1.0 + np.cos(np.pi * ((x - 1.0) / half + 1.0)))
        w = np.where(x < half, left, np.where(x > 1.0 - half, right, 1.0))
        return np.where(inside, w, 0.0)
