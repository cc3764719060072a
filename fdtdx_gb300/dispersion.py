"""Dispersive materials: Lorentz and Drude poles of the auxiliary-differential-equation (ADE)
model (fdtdx/dispersion.py:220-888).

Each pole is a 2nd-order oscillator p'' + gamma p' + omega_0^2 p = K E driven by the field;
its susceptibility is chi(omega) = K / (omega_0^2 - omega^2 - i gamma omega) (the exp(-i
omega t) convention), with K = delta_eps omega_0^2 for a Lorentz pole and K = omega_p^2,
omega_0 = 0 for a Drude pole.  Parameters are scalars (isotropic) or (x, y, z) tuples
(diagonally anisotropic).  Discretised with central differences the polarisation follows
p^{n+1} = c1 p^n + c2 p^{n-1} + c3 E^n with D = 1 + gamma dt / 2,
c1 = (2 - omega_0^2 dt^2) / D, c2 = -(1 - gamma dt / 2) / D, c3 = K dt^2 / D.

The GB300 kernels run the ADE update in forward steps (``k_ade`` before each E half-step);
reverse steps and the reversible gradient refuse dispersive scenes, as the reference's
reversible path does.  Sources see the medium at their carrier (``effective_inv_permittivity``)
and plane sources inject the E side with a broadband impedance-corrected profile
(``dispersive_h_filter``).  Oriented poles and complex pole-residue (CCPR) poles are not
provided.
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


def susceptibility_from_coefficients(c1, c2, c3, omega: float, dt: float) -> np.ndarray:
    """chi(omega) per cell, summed over the leading pole axis, recovered from the stored
    recurrence coefficients (fdtdx/dispersion.py:988-1066, no dE/dt term): with D = 1 + gamma
    dt / 2, gamma dt = 2 (1 + c2) / (1 - c2), omega_0^2 dt^2 = 2 - c1 D and K dt^2 = c3 D, each
    pole gives K / (omega_0^2 - omega^2 - i gamma omega); cells without a pole give 0."""
    c1, c2, c3 = (np.asarray(x, dtype=np.float64) for x in (c1, c2, c3))
    pole = (c1 != 0.0) | (c3 != 0.0)
    one_m = 1.0 - c2
    gdt = np.where(pole, 2.0 * (1.0 + c2) / np.where(one_m == 0.0, 1.0, one_m), 0.0)
    half = 1.0 + 0.5 * gdt
    w0dt2 = np.where(pole, 2.0 - c1 * half, 0.0)
    kdt2 = np.where(pole, c3 * half, 0.0)
    wdt = omega * dt
    den = w0dt2 - wdt * wdt - 1j * gdt * wdt
    return np.where(pole, kdt2 / np.where(pole, den, 1.0), 0.0).sum(axis=0)


def effective_inv_permittivity(inv_eps, c1, c2, c3, omega: float, dt: float) -> np.ndarray:
    """1 / (eps_inf + Re chi(omega)) per cell (fdtdx/dispersion.py:1254-1307): what sources see
    of a dispersive medium at their carrier.  ``inv_eps`` is (1 | 3, *cells), the coefficients
    (poles, 1 | 3, *cells); the result broadcasts the two component axes."""
    chi = susceptibility_from_coefficients(c1, c2, c3, omega, dt)
    return 1.0 / (1.0 / np.asarray(inv_eps, dtype=np.float64) + chi.real)


def eps_spectrum(c1, c2, c3, inv_eps_inf, omegas, dt: float) -> np.ndarray:
    """Slice-averaged eps(omega) = eps_inf + chi(omega) at each angular frequency
    (compute_eps_spectrum_from_coefficients, fdtdx/dispersion.py:1067-1177): per cell eps_inf is
    the component mean of 1 / inv_eps_inf and chi the component mean of the pole sum, then the
    uniform mean over the cells.  Cells are grouped by their coefficients first (a source slice
    holds a handful of materials), so a long spectrum costs one evaluation per material."""
    c1, c2, c3 = (np.asarray(x, dtype=np.float64) for x in (c1, c2, c3))
    P, nd = c1.shape[:2]
    eps_inf = (1.0 / np.asarray(inv_eps_inf, dtype=np.float64)).reshape(np.shape(inv_eps_inf)[0], -1).mean(axis=0)
    rows = np.concatenate([c.reshape(P * nd, -1) for c in (c1, c2, c3)] + [eps_inf[None]], axis=0).T
    uniq, counts = np.unique(rows, axis=0, return_counts=True)
    weights = counts / counts.sum()
    omegas = np.asarray(omegas, dtype=np.float64)
    out = np.zeros(omegas.shape, dtype=np.complex128)
    for row, w in zip(uniq, weights):
        cs = [row[q * P * nd:(q + 1) * P * nd].reshape(P, nd, 1) for q in range(3)]
        out += w * (row[-1] + _chi_mean_over_omegas(cs, omegas, dt))
    return out


def _chi_mean_over_omegas(cs, omegas, dt: float) -> np.ndarray:
    """Component mean of the pole-summed chi of one coefficient row at many frequencies."""
    c1, c2, c3 = (c[..., 0] for c in cs)  # (P, nd)
    pole = (c1 != 0.0) | (c3 != 0.0)
    one_m = 1.0 - c2
    gdt = np.where(pole, 2.0 * (1.0 + c2) / np.where(one_m == 0.0, 1.0, one_m), 0.0)
    half = 1.0 + 0.5 * gdt
    w0dt2 = np.where(pole, 2.0 - c1 * half, 0.0)
    kdt2 = np.where(pole, c3 * half, 0.0)
    wdt = (omegas * dt)[:, None, None]
    den = w0dt2[None] - wdt * wdt - 1j * gdt[None] * wdt
    chi = np.where(pole[None], kdt2[None] / np.where(pole[None], den, 1.0), 0.0)  # (M, P, nd)
    return chi.sum(axis=1).mean(axis=1)


def dispersive_h_filter(raw: np.ndarray, c1, c2, c3, inv_eps_inf, omega_c: float, dt: float) -> np.ndarray:
    """The broadband impedance-corrected profile that a TFSF plane injects on its E side (its H
    incident field's profile) in a dispersive scene (_build_dispersive_H_filter,
    fdtdx/objects/sources/tfsf.py:21-141, with compute_impedance_corrected_temporal_profile,
    fdtdx/dispersion.py:1180-1251): ``raw`` (the profile at every integer step) filtered by
    G = sqrt(eps(omega) / eps(omega_c)) over a zero-padded FFT of length M = the power of two
    >= 2 T, G = 1 at DC and real at Nyquist; unfiltered when no source cell holds a pole."""
    raw = np.asarray(raw, dtype=np.float64)
    if not np.any(np.asarray(c3) != 0.0):
        return raw
    T = raw.shape[0]
    m = 1
    while m < 2 * T:
        m *= 2
    omegas = 2.0 * np.pi * np.fft.rfftfreq(m, d=dt)
    spec = eps_spectrum(c1, c2, c3, inv_eps_inf, omegas, dt)
    eps_c = complex(eps_spectrum(c1, c2, c3, inv_eps_inf, np.array([omega_c]), dt)[0])
    padded = np.zeros(m)
    padded[:T] = raw
    G = np.sqrt(spec / eps_c)
    G[0] = 1.0
    G[-1] = complex(G[-1].real, 0.0)
    return np.fft.irfft(np.fft.rfft(padded) * G, n=m)[:T]
