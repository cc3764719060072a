"""Dispersive materials: Lorentz and Drude poles of the auxiliary-differential-equation (ADE)
model (fdtdx/dispersion.py:220-888).

Each pole is a 2nd-order oscillator p'' + gamma p' + omega_0^2 p = K E driven by the field;
its susceptibility is chi(omega) = K / (omega_0^2 - omega^2 - i gamma omega) (the exp(-i
omega t) convention), with K = delta_eps omega_0^2 for a Lorentz pole and K = omega_p^2,
omega_0 = 0 for a Drude pole.  Parameters are scalars (isotropic) or (x, y, z) tuples
(diagonally anisotropic).  Discretised with central differences the polarisation follows
p^{n+1} = c1 p^n + c2 p^{n-1} + c3 E^n with D = 1 + gamma dt / 2,
c1 = (2 - omega_0^2 dt^2) / D, c2 = -(1 - gamma dt / 2) / D, c3 = K dt^2 / D.

The GB300 kernels do not run dispersive materials yet: a scene that holds one is refused
before any device work.  The models let scenes written for fdtdx construct and give the
oracle the coefficients of the ADE update it states.  Oriented poles and complex
pole-residue (CCPR) poles are not provided.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def _axes(v) -> tuple[float, float, float]:
    if isinstance(v, (int, float)):
        return (float(v),) * 3
    t = tuple(float(x) for x in v)
    if len(t) != 3:
        raise ValueError(f"a pole parameter is a scalar or an (x, y, z) tuple, got {v!r}")
    return t  # type: ignore[return-value]


@dataclass(frozen=True)
class LorentzPole:
    """chi = delta_epsilon omega_0^2 / (omega_0^2 - omega^2 - i gamma omega) (dispersion.py:372-414)."""

    resonance_frequency: float | tuple[float, float, float]
    damping: float | tuple[float, float, float]
    delta_epsilon: float | tuple[float, float, float]

    @property
    def omega_0_axes(self) -> tuple[float, float, float]:
        return _axes(self.resonance_frequency)

    @property
    def gamma_axes(self) -> tuple[float, float, float]:
        return _axes(self.damping)

    @property
    def coupling_sq_axes(self) -> tuple[float, float, float]:
        w, de = self.omega_0_axes, _axes(self.delta_epsilon)
        return (de[0] * w[0] ** 2, de[1] * w[1] ** 2, de[2] * w[2] ** 2)

    @property
    def is_isotropic(self) -> bool:
        return all(len(set(a)) == 1 for a in (self.omega_0_axes, self.gamma_axes, self.coupling_sq_axes))


@dataclass(frozen=True)
class DrudePole:
    """chi = -omega_p^2 / (omega^2 + i gamma omega), a Lorentz pole with omega_0 = 0
    (dispersion.py:417-456)."""

    plasma_frequency: float | tuple[float, float, float]
    damping: float | tuple[float, float, float]

    @property
    def omega_0_axes(self) -> tuple[float, float, float]:
        return (0.0, 0.0, 0.0)

    @property
    def gamma_axes(self) -> tuple[float, float, float]:
        return _axes(self.damping)

    @property
    def coupling_sq_axes(self) -> tuple[float, float, float]:
        wp = _axes(self.plasma_frequency)
        return (wp[0] ** 2, wp[1] ** 2, wp[2] ** 2)

    @property
    def is_isotropic(self) -> bool:
        return all(len(set(a)) == 1 for a in (self.gamma_axes, self.coupling_sq_axes))


@dataclass(frozen=True)
class DispersionModel:
    """A sum of poles (dispersion.py:576-788)."""

    poles: tuple = ()

    @property
    def num_poles(self) -> int:
        return len(self.poles)

    @property
    def is_isotropic(self) -> bool:
        return all(p.is_isotropic for p in self.poles)

    def susceptibility_axes(self, omega: float) -> tuple[complex, complex, complex]:
        out = [0j, 0j, 0j]
        for p in self.poles:
            w0, g, k = p.omega_0_axes, p.gamma_axes, p.coupling_sq_axes
            for ax in range(3):
                out[ax] += k[ax] / (w0[ax] ** 2 - omega**2 - 1j * g[ax] * omega)
        return (out[0], out[1], out[2])

    def susceptibility(self, omega: float) -> complex:
        if not self.is_isotropic:
            raise ValueError("the model has per-axis poles; use susceptibility_axes")
        return self.susceptibility_axes(omega)[0]


def compute_pole_coefficients_per_axis(poles, dt: float) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """(c1, c2, c3, c4), each (len(poles), 3), of the ADE recurrence (dispersion.py:789-857),
    the reference's four arrays; c4 (the term of a pole with a numerator coefficient b) is
    zero for the Lorentz and Drude poles here.  A coupled axis needs omega_0 dt < 2 for the
    recurrence to stay stable."""
    n = len(poles)
    c1, c2, c3, c4 = (np.zeros((n, 3)) for _ in range(4))
    for i, p in enumerate(poles):
        w0, g, k = p.omega_0_axes, p.gamma_axes, p.coupling_sq_axes
        for ax in range(3):
            if k[ax] != 0.0 and w0[ax] * dt >= 2.0:
                raise ValueError(f"pole {i}: omega_0 * dt = {w0[ax] * dt:.4g} >= 2 makes the ADE recurrence unstable")
            d = 1.0 + 0.5 * g[ax] * dt
            c1[i, ax] = (2.0 - w0[ax] ** 2 * dt**2) / d
            c2[i, ax] = -(1.0 - 0.5 * g[ax] * dt) / d
            c3[i, ax] = k[ax] * dt**2 / d
    return c1, c2, c3, c4
