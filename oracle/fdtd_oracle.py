"""ORACLE -- test infrastructure only.  CPU restatement of fdtdx's time-stepping path.

This module is the checker of the GB300 library: only ``tests/``, the smoke test
of ``__graft_entry__`` and the CPU-baseline leg of ``bench.py`` may import it.
The product path (``fdtdx_gb300``) never calls it.

It restates, line by line in torch-CPU tensors (so that the same code runs in
float64 for the error reference, in float32 for the parity reference, and under
torch autograd for per-step vector-Jacobian products), the reference files:

* fdtdx/fdtd/update.py:256-1007       update_E / update_H and their reverses
* fdtdx/core/physics/curl.py:86-397   curls with CPML corrections, co-location
* fdtdx/core/misc.py:615-641          halo padding
* fdtdx/fdtd/update.py:92-136, objects/boundaries/bloch.py:13-155, fdtd/initialization.py:581-594
                                      Bloch ghost-layer phases and complex fields
* fdtdx/objects/boundaries/perfectly_matched_layer.py:69-275   CPML coefficients
* fdtdx/objects/boundaries/pec.py:71-77, pmc.py:62-76          conductor walls
* fdtdx/objects/sources/dipole.py:150-277                      point dipole
* fdtdx/objects/sources/profile.py:253-345, core/window.py:16-30  temporal profiles
* fdtdx/objects/sources/linear_polarization.py:168-468, tfsf.py:144-409, 739-806,
  fdtdx/core/grid.py:720-880                                   TFSF plane source
* fdtdx/fdtd/update.py:316-350, dispersion.py:789-857, 988-1066, 1067-1251, 1254-1307,
  fdtd/initialization.py:686-1000, tfsf.py:21-141, 256-261   dispersive (ADE) Lorentz / Drude
  poles: coefficients, update, carrier-frequency sources and the H-side impedance filter
* fdtdx/core/linalg.py:50-160, core/misc.py:363-390, 508-553   source tilt (dipole
  orientation, tilted plane polarisation, projection and bilinear sampling)
* fdtdx/objects/detectors/{detector,phasor,field,poynting_flux,energy}.py  detectors
* fdtdx/fdtd/update.py:1040-1222, fdtdx/fdtd/misc.py:10-66     detectors, interfaces
* fdtdx/fdtd/forward.py:83-156, backward.py:62-135, fdtd.py:39-418  step and VJP loop
* fdtdx/fdtd/update.py:356-523, 641-676, 751-807, 956-995, fdtdx/fdtd/misc.py:69-213,
  fdtdx/core/misc.py:557-611   full 3x3 anisotropic update branch (uniform grid), with
  the tensor branches of the sources (dipole.py:15-37, tfsf.py:144-190, 287-299, 384-393)
  and of the energy detector (core/physics/metrics.py:34-51); the GB300 library does not
  build this branch yet, the oracle states it for its pins

Parity status: the reference is JAX and JAX cannot be installed on these machines,
so the reference itself cannot be run.  The reference's tests hold no stored field
or detector values; what they hold are known-answer tests and invariants (curl of
a linear field, CPML scatter signs, update formulas, forward/backward round trips,
PML profile values, phasor semantics), and those are replayed against this oracle
in tests/test_oracle_kats.py, together with the reference's simulation-tier physics
checks (analytic wavenumbers, impedances, Fresnel coefficients, skin depth, radiation
patterns, dispersion, Bloch oblique incidence) in tests/test_oracle_physics.py,
test_tilted_sources.py, test_oracle_bloch.py, test_oracle_dispersion.py and
test_oracle_aniso.py, and its gradient checks in tests/test_oracle_gradient.py.  Beyond
those, field-level parity is unpinned.

Objects are read through their fdtdx attribute names (duck typing), so a scene
built with ``fdtdx_gb300`` objects drives this oracle without using any of that
package's setup code.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any

import numpy as np
import torch

C0 = 299792458.0
MU0 = 4e-7 * math.pi
EPS0 = 1.0 / (MU0 * C0**2)
ETA0 = MU0 * C0
COMPONENTS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


def jax_index(n: int, t: int) -> int:
    """Index of a length-n array read at t by a JAX gather: negative wraps, overflow clamps."""
    if t < 0:
        t += n
    return min(max(t, 0), n - 1)


# --------------------------------------------------------------------------------------------
# padding and curls
# --------------------------------------------------------------------------------------------


def pad_fields(f: torch.Tensor, periodic: tuple[bool, bool, bool], bloch=()) -> torch.Tensor:
    """One-cell halo per axis, wrap or zero, applied axis by axis (fdtdx/core/misc.py:615-641),
    then the Bloch ghost-cell phases (fdtdx/fdtd/update.py:92-136,
    objects/boundaries/bloch.py:59-94): for each (axis, direction, phase) of a Bloch boundary
    with a non-zero vector, the '-' ghost layer (wrapped from the far end) is multiplied by
    conj(phase) and the '+' ghost layer by phase, phase = exp(i k L)."""
    for ax, per in enumerate(periodic):
        d = ax + 1
        n = f.shape[d]
        if per:
            lo, hi = f.narrow(d, n - 1, 1), f.narrow(d, 0, 1)
        else:
            z = torch.zeros_like(f.narrow(d, 0, 1))
            lo, hi = z, z
        f = torch.cat([lo, f, hi], dim=d)
    for ax, direction, phase in bloch:
        f = f.clone()
        idx = [slice(None)] * f.dim()
        idx[ax + 1] = 0 if direction == "-" else -1
        f[tuple(idx)] = f[tuple(idx)] * (phase.conj() if direction == "-" else phase)
    return f


def _add_at(a: torch.Tensor, sl, v) -> torch.Tensor:
    out = a.clone()
    out[sl] = out[sl] + v
    return out


def _set_at(a: torch.Tensor, sl, v) -> torch.Tensor:
    out = a.clone()
    out[sl] = v
    return out


@dataclass
class OPml:
    name: str
    axis: int
    direction: str
    grid_slice: tuple
    kappa_start: float
    kappa_end: float
    a_E: torch.Tensor
    b_E: torch.Tensor
    inv_kappa_E: torch.Tensor
    a_H: torch.Tensor
    b_H: torch.Tensor
    inv_kappa_H: torch.Tensor


def pml_coefficients(pml, dx: float, dt: float, dtype) -> dict[str, torch.Tensor]:
    """perfectly_matched_layer.py:97-136 and _compute_pml_profile :231-275 (uniform grid)."""
    L = pml.grid_shape[pml.axis]
    sigma_end = pml.sigma_end
    if sigma_end is None:
        sigma_end = -(pml.sigma_order + 1) * math.log(1e-6) / (2 * (ETA0 / 1.0) * (L * dx))
    if pml.direction == "-":
        dE = np.arange(L - 1, -1, -1, dtype=np.float64)
        dH = np.append(np.arange(L - 1.5, -0.5, -1, dtype=np.float64), 0)
    else:
        dE = np.insert(np.arange(0.5, L - 0.5, 1, dtype=np.float64), 0, 0)
        dH = np.arange(0, L, 1, dtype=np.float64)
    dE = torch.tensor(dE, dtype=dtype)
    dH = torch.tensor(dH, dtype=dtype)

    def profile(v0, v1, order):
        return v0 + (v1 - v0) * torch.pow(dE / L, order), v0 + (v1 - v0) * torch.pow(dH / L, order)

    sigma_E, sigma_H = profile(pml.sigma_start, sigma_end, pml.sigma_order)
    kappa_E, kappa_H = profile(pml.kappa_start, pml.kappa_end, pml.kappa_order)
    alpha_E, alpha_H = profile(pml.alpha_start, pml.alpha_end, pml.alpha_order)
    b_E = torch.expm1(-dt / EPS0 * (sigma_E / kappa_E + alpha_E)) + 1
    a_E = torch.nan_to_num((b_E - 1.0) * sigma_E / (sigma_E + alpha_E * kappa_E) / kappa_E, nan=0.0)
    b_H = torch.expm1(-dt / EPS0 * (sigma_H / kappa_H + alpha_H)) + 1
    a_H = torch.nan_to_num((b_H - 1.0) * sigma_H / (sigma_H + alpha_H * kappa_H) / kappa_H, nan=0.0)
    shape = [1, 1, 1]
    shape[pml.axis] = L
    return {
        "a_E": a_E.reshape(shape), "b_E": b_E.reshape(shape), "inv_kappa_E": (1.0 / kappa_E).reshape(shape),
        "a_H": a_H.reshape(shape), "b_H": b_H.reshape(shape), "inv_kappa_H": (1.0 / kappa_H).reshape(shape),
        "sigma_end": sigma_end,
    }


def step_cpml(pml: OPml, d1, d2, psi1, psi2, is_curl_E: bool, simulate_boundaries: bool):
    """perfectly_matched_layer.py:138-190."""
    if is_curl_E:
        a, b, ik = pml.a_H, pml.b_H, pml.inv_kappa_H
    else:
        a, b, ik = pml.a_E, pml.b_E, pml.inv_kappa_E
    if simulate_boundaries:
        p1 = b * psi1 + a * d1
        p2 = b * psi2 + a * d2
    else:
        p1, p2 = psi1, psi2
    if pml.kappa_start == 1.0 and pml.kappa_end == 1.0:
        c1, c2 = p1, p2
    else:
        c1 = (ik - 1.0) * d1 + p1
        c2 = (ik - 1.0) * d2 + p2
    return c1, c2, p1, p2


def curl_E(E_pad, psi_H, pmls, simulate_boundaries):
    """fdtdx/core/physics/curl.py:227-311 (uniform grid: metric scale 1)."""
    Ex, Ey, Ez = E_pad[0], E_pad[1], E_pad[2]
    c = (slice(1, -1), slice(1, -1), slice(1, -1))
    dyEz = Ez[1:-1, 2:, 1:-1] - Ez[c]
    dzEy = Ey[1:-1, 1:-1, 2:] - Ey[c]
    dzEx = Ex[1:-1, 1:-1, 2:] - Ex[c]
    dxEz = Ez[2:, 1:-1, 1:-1] - Ez[c]
    dxEy = Ey[2:, 1:-1, 1:-1] - Ey[c]
    dyEx = Ex[1:-1, 2:, 1:-1] - Ex[c]
    comps = [dyEz - dzEy, dzEx - dxEz, dxEy - dyEx]
    new_psi = {}
    for pml in pmls:
        a = pml.axis
        i, j = (a + 1) % 3, (a + 2) % 3
        if a == 0:
            dj, di = dxEz, dxEy
        elif a == 1:
            dj, di = dyEx, dyEz
        else:
            dj, di = dzEy, dzEx
        gs = pml.grid_slice
        p1, p2 = psi_H[pml.name]
        c1, c2, p1n, p2n = step_cpml(pml, dj[gs], di[gs], p1, p2, True, simulate_boundaries)
        comps[i] = _add_at(comps[i], gs, -c1)
        comps[j] = _add_at(comps[j], gs, c2)
        new_psi[pml.name] = (p1n, p2n)
    return torch.stack(comps, 0), new_psi


def curl_H(H_pad, psi_E, pmls, simulate_boundaries):
    """fdtdx/core/physics/curl.py:314-397 (uniform grid)."""
    Hx, Hy, Hz = H_pad[0], H_pad[1], H_pad[2]
    c = (slice(1, -1), slice(1, -1), slice(1, -1))
    dyHz = Hz[c] - Hz[1:-1, :-2, 1:-1]
    dzHy = Hy[c] - Hy[1:-1, 1:-1, :-2]
    dzHx = Hx[c] - Hx[1:-1, 1:-1, :-2]
    dxHz = Hz[c] - Hz[:-2, 1:-1, 1:-1]
    dxHy = Hy[c] - Hy[:-2, 1:-1, 1:-1]
    dyHx = Hx[c] - Hx[1:-1, :-2, 1:-1]
    comps = [dyHz - dzHy, dzHx - dxHz, dxHy - dyHx]
    new_psi = {}
    for pml in pmls:
        a = pml.axis
        i, j = (a + 1) % 3, (a + 2) % 3
        if a == 0:
            dj, di = dxHz, dxHy
        elif a == 1:
            dj, di = dyHx, dyHz
        else:
            dj, di = dzHy, dzHx
        gs = pml.grid_slice
        p1, p2 = psi_E[pml.name]
        c1, c2, p1n, p2n = step_cpml(pml, dj[gs], di[gs], p1, p2, False, simulate_boundaries)
        comps[i] = _add_at(comps[i], gs, -c1)
        comps[j] = _add_at(comps[j], gs, c2)
        new_psi[pml.name] = (p1n, p2n)
    return torch.stack(comps, 0), new_psi


def interpolate_fields(E_pad, H_pad):
    """Co-location at the E_z point (i, j, k+1/2), fdtdx/core/physics/curl.py:86-224 (uniform grid)."""
    Ex, Ey, Ez = E_pad[0], E_pad[1], E_pad[2]
    Hx, Hy, Hz = H_pad[0], H_pad[1], H_pad[2]

    def avg(cur, prev):
        return 0.5 * (cur + prev)

    Ex_lo = avg(Ex[1:-1, 1:-1, 1:-1], Ex[:-2, 1:-1, 1:-1])
    Ex_up = avg(Ex[1:-1, 1:-1, 2:], Ex[:-2, 1:-1, 2:])
    ex = (Ex_lo + Ex_up) / 2.0
    Ey_lo = avg(Ey[1:-1, 1:-1, 1:-1], Ey[1:-1, :-2, 1:-1])
    Ey_up = avg(Ey[1:-1, 1:-1, 2:], Ey[1:-1, :-2, 2:])
    ey = (Ey_lo + Ey_up) / 2.0
    ez = Ez[1:-1, 1:-1, 1:-1]
    hx = avg(Hx[1:-1, 1:-1, 1:-1], Hx[1:-1, :-2, 1:-1])
    hy = avg(Hy[1:-1, 1:-1, 1:-1], Hy[:-2, 1:-1, 1:-1])
    lx = avg(Hz[1:-1, 1:-1, 1:-1], Hz[:-2, 1:-1, 1:-1])
    lxy = avg(lx, avg(Hz[1:-1, :-2, 1:-1], Hz[:-2, :-2, 1:-1]))
    ux = avg(Hz[1:-1, 1:-1, 2:], Hz[:-2, 1:-1, 2:])
    uxy = avg(ux, avg(Hz[1:-1, :-2, 2:], Hz[:-2, :-2, 2:]))
    hz = (lxy + uxy) / 2.0
    return torch.stack([ex, ey, ez], 0), torch.stack([hx, hy, hz], 0)


# --------------------------------------------------------------------------------------------
# temporal profiles
# --------------------------------------------------------------------------------------------


def profile_amplitude(profile, time: torch.Tensor, period: float, phase_shift: float) -> torch.Tensor:
    """fdtdx/objects/sources/profile.py:253-345 with core/window.py:16-30 (Re(exp(-i p)) = cos p)."""
    name = type(profile).__name__
    if name == "SingleFrequencyProfile":
        phase = 2 * math.pi * time / period + phase_shift + profile.phase_shift
        raw = torch.cos(phase)
        factor = torch.clamp(time / (profile.num_startup_periods * period), 0.0, 1.0)
        return factor * raw
    if name == "GaussianPulseProfile":
        sigma_t = 1.0 / (2 * math.pi * profile.spectral_width.get_frequency())
        t0 = 6 * sigma_t
        env = torch.exp(-((time - t0) ** 2) / (2.0 * sigma_t**2))
        phase = 2 * math.pi * profile.center_wave.get_frequency() * time + phase_shift + profile.center_wave.phase_shift
        return env * torch.cos(phase)
    raise NotImplementedError(name)


# --------------------------------------------------------------------------------------------
# scene
# --------------------------------------------------------------------------------------------


def tilt_vector(vec: torch.Tensor, azimuth: float, elevation: float, axes: tuple[int, int, int]) -> torch.Tensor:
    """rotate_vector (fdtdx/core/linalg.py:90-160, rotation matrices :50-87): global -> raw
    basis (rows e_h, e_v, e_p), through the rows u = R_1(azimuth) e1, v = R_0(elevation) e2,
    w = u x v / |u x v|, back to global, rescaled to the input's norm."""
    dt_ = vec.dtype
    h_ax, v_ax, p_ax = axes
    eye = torch.eye(3, dtype=dt_)
    to_raw = torch.stack((eye[h_ax], eye[v_ax], eye[p_ax]), 0)
    ca, sa = math.cos(azimuth), math.sin(azimuth)
    ce, se = math.cos(elevation), math.sin(elevation)
    az_m = torch.tensor([[ca, 0.0, -sa], [0.0, 1.0, 0.0], [sa, 0.0, ca]], dtype=dt_)
    el_m = torch.tensor([[1.0, 0.0, 0.0], [0.0, ce, -se], [0.0, se, ce]], dtype=dt_)
    u = az_m @ torch.tensor([1.0, 0.0, 0.0], dtype=dt_)
    v = el_m @ torch.tensor([0.0, 1.0, 0.0], dtype=dt_)
    w = torch.linalg.cross(u, v)
    w = w / torch.linalg.norm(w)
    rotated = torch.stack((u, v, w), 0) @ (to_raw @ vec)
    out = to_raw.T @ rotated
    return out / torch.linalg.norm(out) * torch.linalg.norm(vec)


def linear_interpolated_indexing(points: torch.Tensor, arr: torch.Tensor) -> torch.Tensor:
    """fdtdx/core/misc.py:363-390 for a batch of 2-D points (P, 2): the floor / ceil corners,
    weights prod(1 - |corner - point|), corners outside ``arr`` weighted 0 (and read at 0), and
    sum(w v) / (sum(w) + 1e-8)."""
    fl, ce = torch.floor(points), torch.ceil(points)
    num = torch.zeros(points.shape[0], dtype=arr.dtype)
    den = torch.zeros(points.shape[0], dtype=arr.dtype)
    for c0 in (fl[:, 0], ce[:, 0]):
        for c1 in (fl[:, 1], ce[:, 1]):
            corner = torch.stack((c0, c1), -1)
            wgt = (1 - (corner - points).abs()).prod(-1)
            bad = (c0 < 0) | (c0 >= arr.shape[0]) | (c1 < 0) | (c1 >= arr.shape[1])
            wgt = torch.where(bad, torch.zeros_like(wgt), wgt)
            i0 = torch.where(bad, torch.zeros_like(c0), c0).long()
            i1 = torch.where(bad, torch.zeros_like(c1), c1).long()
            num = num + wgt * arr[i0, i1]
            den = den + wgt
    return num / (den + 1e-8)


def _chi_from_coefficients(c1, c2, c3, omega: float, dt: float) -> torch.Tensor:
    """susceptibility_from_coefficients (dispersion.py:988-1066) without the dE/dt coupling,
    summed over the pole axis; cells whose coefficients are all zero give 0."""
    mask = (c1 != 0) | (c3 != 0)
    omc2 = 1.0 - c2
    gdt = torch.where(mask, 2.0 * (1.0 + c2) / torch.where(omc2 == 0, torch.ones_like(omc2), omc2),
                      torch.zeros_like(c2))
    half = 1.0 + 0.5 * gdt
    w0dt2 = torch.where(mask, 2.0 - c1 * half, torch.zeros_like(c1))
    adt2 = torch.where(mask, c3 * half, torch.zeros_like(c3))
    wdt = omega * dt
    den = w0dt2 - wdt * wdt - 1j * gdt * wdt
    chi = torch.where(mask, adt2 / torch.where(mask, den, torch.ones_like(den)), torch.zeros_like(den))
    return chi.sum(0)


@dataclass
class OSource:
    obj: Any
    kind: str
    on: list
    on_idx: list
    default_on: bool
    # dipole
    inv_local: torch.Tensor | None = None
    orient: torch.Tensor | None = None
    # plane
    E_inc: torch.Tensor | None = None
    H_inc: torch.Tensor | None = None
    off_E: torch.Tensor | None = None
    off_H: torch.Tensor | None = None
    h_filter: np.ndarray | None = None  # H-side profile at integer steps in dispersive scenes


@dataclass
class ODetector:
    obj: Any
    kind: str
    on: list
    arr_idx: list
    window: np.ndarray | None = None
    scale: float = 1.0


class OracleScene:
    """A placed scene restated for the oracle in one dtype (float32 or float64)."""

    def __init__(self, objects, arrays, config, dtype=torch.float64):
        self.dtype = dtype
        vol = objects.volume
        self.shape = tuple(vol.grid_shape)
        self.dx = float(config.grid.spacing)
        self.courant = config.courant_factor / math.sqrt(3)
        self.dt = self.courant * self.dx / C0
        self.T = round(config.time / self.dt)
        self.inv_eps = arrays.inv_permittivities.detach().to("cpu", dtype)
        mu = arrays.inv_permeabilities
        self.inv_mu = mu.detach().to("cpu", dtype) if isinstance(mu, torch.Tensor) else float(mu)
        se, sh = arrays.electric_conductivity, arrays.magnetic_conductivity
        self.sigma_E = se.detach().to("cpu", dtype) if se is not None else None
        self.sigma_H = sh.detach().to("cpu", dtype) if sh is not None else None
        self.periodic = [False, False, False]
        self.pec, self.pmc, self.pmls = [], [], []
        self.bloch = []  # (axis, direction, exp(i k L)) of Bloch boundaries with k != 0
        cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
        for b in objects.boundary_objects:
            name = type(b).__name__
            if name in ("PeriodicBoundary", "BlochBoundary"):
                self.periodic[b.axis] = True
                k = float(getattr(b, "bloch_vector", (0.0, 0.0, 0.0))[b.axis])
                if k != 0.0:  # get_bloch_phase (bloch.py:133-155), uniform grid
                    L = self.shape[b.axis] * self.dx
                    self.bloch.append((b.axis, b.direction, torch.exp(torch.tensor(1j * k * L, dtype=cdt))))
            elif name == "PerfectElectricConductor":
                self.pec.append(b)
            elif name == "PerfectMagneticConductor":
                self.pmc.append(b)
            elif name == "PerfectlyMatchedLayer":
                co = pml_coefficients(b, self.dx, self.dt, dtype)
                self.pmls.append(
                    OPml(b.name, b.axis, b.direction, b.grid_slice, b.kappa_start, b.kappa_end, co["a_E"], co["b_E"],
                         co["inv_kappa_E"], co["a_H"], co["b_H"], co["inv_kappa_H"])
                )
        self.periodic = tuple(self.periodic)
        # complex fields exactly when a Bloch vector is non-zero (fdtd/initialization.py:581-594)
        self.field_dtype = cdt if self.bloch else dtype
        self.disp = self._setup_dispersion(objects)
        self.sources = [self._setup_source(s) for s in objects.sources]
        self.detectors = [self._setup_detector(d) for d in objects.detectors if not d.inverse]
        self._setup_time_filter(config)

    # ---- recorder time filter (fdtdx/interfaces/time_filter.py:140-257)
    def _setup_time_filter(self, config):
        self.tf_save, self.tf_map = None, None
        gc = getattr(config, "gradient_config", None)
        rec = getattr(gc, "recorder", None) if gc is not None else None
        for m in getattr(rec, "modules", []) if rec is not None else []:
            if type(m).__name__ != "LinearReconstructEveryK":
                continue
            T, k = self.T, m.k
            save = list(range(m.start_recording_after, T, k))  # time_filter.py:168-171
            if save[-1] != T - 1:
                save.append(T - 1)
            idx = np.zeros(T, dtype=np.int64)  # time_filter.py:176-187
            idx[save] = np.arange(len(save))
            for _ in range(k - 1):
                rolled = np.roll(idx, 1)
                idx = np.where(idx == 0, rolled, idx)
                idx[:k] = 0
            self.tf_save, self.tf_map = save, idx

    def recorded(self, rec: list, t: int) -> dict:
        """Interface values the reverse step at t re-imposes (time_filter.py:218-257)."""
        if self.tf_save is None:
            return rec[t]  # a Python list wraps t = -1 like the JAX gather
        tj = t + self.T if t < 0 else t
        a = int(self.tf_map[tj])
        if tj in self.tf_save:
            return rec[a]
        nxt = min(a + 1, len(rec) - 1)  # a JAX gather clamps the index
        t_prev = int(np.argmax(self.tf_map == a))  # index_1d_array: first step mapped to the slot
        t_next = int(np.argmax(self.tf_map == a + 1))
        f = (t - t_prev) / (t_next - t_prev)
        return {key: v + f * (rec[nxt][key] - v) for key, v in rec[a].items()}

    def records(self, t: int) -> bool:
        return self.tf_save is None or t in self.tf_save

    # ---- dispersion
    def _setup_dispersion(self, objects):
        """Per-cell ADE coefficients (c1, c2, c3), each (poles, 1 | 3, *grid), or None without
        dispersive materials (fdtd/initialization.py:686-700, 795-830, 955-1000): every painted
        material, the volume first and then the material objects in placement order, writes its
        pole stack over its slice, zero-padded to the scene's pole count (zeros for a material
        without poles); one component when every pole is isotropic, else three.  Coefficients
        of dispersion.py:789-857; stored in the scene dtype."""
        painted = [objects.volume] + sorted(objects.static_material_objects, key=lambda o: o.placement_order)
        mats = [(o, getattr(o, "material", None)) for o in painted]
        models = [m.dispersion for _, m in mats
                  if m is not None and getattr(m, "dispersion", None) is not None and m.dispersion.num_poles > 0]
        if not models:
            return None
        n_poles = max(d.num_poles for d in models)
        nc = 1 if all(d.is_isotropic for d in models) else 3
        cs = [torch.zeros((n_poles, nc, *self.shape), dtype=torch.float64) for _ in range(3)]
        for o, m in mats:
            if m is None:
                continue
            poles = m.dispersion.poles if getattr(m, "dispersion", None) is not None else ()
            block = [torch.zeros((n_poles, nc), dtype=torch.float64) for _ in range(3)]
            for i, p in enumerate(poles):
                if getattr(p, "orientation", None) is not None or any(getattr(p, "coupling_edot_axes", (0.0,) * 3)):
                    raise NotImplementedError("oriented and CCPR poles")
                w0, g, k = p.omega_0_axes, p.gamma_axes, p.coupling_sq_axes
                for ax in range(nc):
                    if k[ax] != 0.0 and w0[ax] * self.dt >= 2.0:
                        raise ValueError("omega_0 * dt >= 2: the ADE recurrence is unstable")
                    den = 1.0 + 0.5 * g[ax] * self.dt
                    block[0][i, ax] = (2.0 - w0[ax] ** 2 * self.dt**2) / den
                    block[1][i, ax] = -(1.0 - 0.5 * g[ax] * self.dt) / den
                    block[2][i, ax] = k[ax] * self.dt**2 / den
            for c, b in zip(cs, block):
                c[(slice(None), slice(None), *o.grid_slice)] = b[:, :, None, None, None]
        return tuple(c.to(self.dtype) for c in cs)

    def _eff_inv_eps(self, inv_eps_slice, sl, omega: float):
        """effective_inv_permittivity (dispersion.py:988-1066, 1254-1307): 1 / (eps_inf +
        Re chi(omega)) per cell, chi from the stored coefficients by inverting the recurrence
        (gamma dt = 2 (1 + c2) / (1 - c2), omega_0^2 dt^2 = 2 - c1 D, K dt^2 = c3 D), cells
        without a pole unchanged."""
        if self.disp is None:
            return inv_eps_slice
        c1, c2, c3 = (c[(slice(None), slice(None), *sl)].to(torch.float64) for c in self.disp)
        chi = _chi_from_coefficients(c1, c2, c3, omega, self.dt)  # (1 | 3, *slice)
        return (1.0 / (1.0 / inv_eps_slice.to(torch.float64) + chi.real)).to(inv_eps_slice.dtype)

    def _h_filter(self, s) -> np.ndarray:
        """_build_dispersive_H_filter (tfsf.py:21-141) with
        compute_eps_spectrum_from_coefficients (dispersion.py:1067-1177) and
        compute_impedance_corrected_temporal_profile (dispersion.py:1180-1251): the raw profile
        sampled at every integer step; unless the source cells hold no pole, filtered by
        G = sqrt(eps(omega) / eps(omega_c)) (slice-averaged eps, G = 1 at DC, real at Nyquist)
        over a zero-padded FFT of length M = the power of two >= 2 T."""
        T = self.T
        raw = np.array([float(profile_amplitude(s.temporal_profile, torch.tensor(n * self.dt, dtype=torch.float64),
                                                s.wave_character.get_period(), s.wave_character.phase_shift))
                        for n in range(T)])
        cs = [c[(slice(None), slice(None), *s.grid_slice)].to(torch.float64) for c in self.disp]
        if not bool(torch.any(cs[2] != 0)):
            return raw
        m = 1
        while m < 2 * T:
            m *= 2
        inv_inf = self.inv_eps[(slice(None), *s.grid_slice)].to(torch.float64)
        eps_inf = (1.0 / inv_inf).mean(0)

        def eps_mean(omega):
            chi = _chi_from_coefficients(cs[0], cs[1], cs[2], omega, self.dt)  # (C, *slice)
            return complex((eps_inf + chi.mean(0)).mean())

        omegas = 2 * np.pi * np.fft.rfftfreq(m, d=self.dt)
        spectrum_eps = np.array([eps_mean(float(w)) for w in omegas])
        eps_c = eps_mean(2 * np.pi * s.wave_character.get_frequency())
        padded = np.zeros(m)
        padded[:T] = raw
        G = np.sqrt(spectrum_eps / eps_c)
        G[0] = 1.0
        G[-1] = complex(G[-1].real, 0.0)
        return np.fft.irfft(np.fft.rfft(padded) * G, n=m)[:T]

    # ---- sources
    def _switch_tables(self, sw):
        on = sw.calculate_on_list(self.T, self.dt)
        idx = sw.calculate_time_step_to_on_arr_idx(self.T, self.dt)
        return on, idx

    def _setup_source(self, s) -> OSource:
        on, idx = self._switch_tables(s.switch)
        default_on = s.switch.is_default_always_on
        name = type(s).__name__
        if name == "PointDipoleSource":
            inv = self.inv_eps if s.source_type == "electric" else self.inv_mu
            if isinstance(inv, torch.Tensor):
                local = inv[(slice(None), *s.grid_slice)]
                if s.source_type == "electric":  # sampled at the carrier in dispersive media (dipole.py:168-180)
                    local = self._eff_inv_eps(local, s.grid_slice, 2 * math.pi * s.wave_character.get_frequency())
            else:
                local = torch.tensor(inv, dtype=self.dtype)
            # _orientation (dipole.py:130-148)
            orient = torch.zeros(3, dtype=self.dtype)
            orient[s.polarization] = 1.0
            if s.azimuth_angle != 0.0 or s.elevation_angle != 0.0:
                p = s.polarization
                orient = tilt_vector(orient, float(np.deg2rad(s.azimuth_angle)), float(np.deg2rad(s.elevation_angle)),
                                     ((p + 1) % 3, (p + 2) % 3, p))
            return OSource(s, "dipole", on, idx, default_on, inv_local=local, orient=orient)
        if name in ("GaussianPlaneSource", "UniformPlaneSource"):
            E, H, oE, oH = self._plane_apply(s)
            return OSource(s, "plane", on, idx, default_on, E_inc=E, H_inc=H, off_E=oE, off_H=oH,
                           h_filter=self._h_filter(s) if self.disp is not None else None)
        raise NotImplementedError(name)

    def _plane_apply(self, s):
        """LinearlyPolarizedPlaneSource.apply on a uniform grid, normal or tilted incidence
        (linear_polarization.py:168-358); no random centre or angle offsets."""
        dt_ = self.dtype
        gs = s.grid_shape
        n = gs.index(1)
        h_ax, v_ax = (n + 1) % 3, (n + 2) % 3
        W, Hh = gs[h_ax], gs[v_ax]
        center = torch.tensor([0.5 * (0 + W - 1), 0.5 * (0 + Hh - 1)], dtype=dt_)
        # polarization (core/misc.py:471-505, core/linalg.py:7-47)
        k = torch.zeros(3, dtype=dt_)
        k[n] = 1.0 if s.direction == "+" else -1.0
        e = None if s.fixed_E_polarization_vector is None else torch.tensor(s.fixed_E_polarization_vector, dtype=dt_)
        h = None if s.fixed_H_polarization_vector is None else torch.tensor(s.fixed_H_polarization_vector, dtype=dt_)
        if h is not None:
            h = h / torch.linalg.norm(h)
        if e is not None:
            e = e / torch.linalg.norm(e)
        if e is None:
            e = torch.linalg.cross(h, k)
        if h is None:
            h = torch.linalg.cross(k, e)
        tilted = s.azimuth_angle != 0.0 or s.elevation_angle != 0.0
        if getattr(s, "max_angle_random_offset", 0.0):
            raise NotImplementedError("random angle offsets")
        if tilted:  # tilted_polarization_vectors (core/misc.py:508-553)
            az, el = float(np.deg2rad(s.azimuth_angle)), float(np.deg2rad(s.elevation_angle))
            e, h, k = (tilt_vector(x, az, el, (h_ax, v_ax, n)) for x in (e, h, k))
        # raw amplitude (linear_polarization.py:392-482)
        if type(s).__name__ == "GaussianPlaneSource":
            r = s.radius / self.dx
            w_, h_ = torch.meshgrid(torch.arange(W, dtype=dt_), torch.arange(Hh, dtype=dt_), indexing="ij")
            grid = (torch.stack([w_, h_], -1) - center) / torch.tensor([r, r], dtype=dt_)
            d2 = (grid**2).sum(-1)
            prof = torch.where(d2 < 1, torch.exp(-0.5 * d2 / s.std**2), torch.zeros_like(d2))
            prof_hv = prof / prof.sum()
        else:
            prof_hv = s.amplitude * torch.ones((W, Hh), dtype=dt_)
        if tilted:
            # projection onto the plane normal to k in the basis (u, v) (linear_polarization.py:241-286)
            e_h = torch.zeros(3, dtype=dt_)
            e_h[h_ax] = 1.0
            ub = e_h - torch.dot(e_h, k) * k
            ub = ub / torch.linalg.norm(ub)
            vb = (1.0 if s.direction == "+" else -1.0) * torch.linalg.cross(k, ub)
            w_, h_ = torch.meshgrid(torch.arange(W, dtype=dt_), torch.arange(Hh, dtype=dt_), indexing="ij")
            wh = (torch.stack([w_, h_], -1) - center).reshape(-1, 2)
            pt = torch.zeros(wh.shape[0], 3, dtype=dt_)
            pt[:, h_ax] = wh[:, 0]
            pt[:, v_ax] = wh[:, 1]
            proj = pt - (pt @ k)[:, None] * k
            fp = torch.stack([proj @ ub, proj @ vb], -1) + center
            interp = linear_interpolated_indexing(fp, prof_hv).reshape(prof_hv.shape)
        else:
            # projection of the untilted plane is the identity; linear_interpolated_indexing at an
            # integer point returns 4 v / (4 + 1e-8) (core/misc.py:363-390)
            interp = (4.0 * prof_hv) / (4.0 + 1e-8)
        prof2 = interp.T if h_ax > v_ax else interp
        amp = prof2.unsqueeze(n)[None]
        E = amp * e[:, None, None, None]
        H = amp * h[:, None, None, None]
        sl = (slice(None), *s.grid_slice)
        # impedance, energy and offsets see the medium at the carrier (linear_polarization.py:186-211)
        ie = self._eff_inv_eps(self.inv_eps[sl], s.grid_slice, 2 * math.pi * s.wave_character.get_frequency())
        im = self.inv_mu[sl] if isinstance(self.inv_mu, torch.Tensor) else self.inv_mu
        full = _is9(ie) or _is9(im)
        if full:  # tensor media: eps = inv(inv_eps) per cell (core/physics/metrics.py:34-51, tfsf.py:144-190)
            eps_t = _tensor_inverse(expand_to_3x3(ie)).to(dt_).expand(3, 3, *gs)
            mu_t = _tensor_inverse(expand_to_3x3(im)).to(dt_).expand(3, 3, *gs)
        if s.normalize_by_energy:
            if full:
                energy = 0.5 * torch.einsum("ixyz,ijxyz,jxyz->xyz", E.conj(), eps_t.to(E.dtype), E).real \
                    + 0.5 * torch.einsum("ixyz,ijxyz,jxyz->xyz", H.conj(), mu_t.to(H.dtype), H).real
            else:
                energy = (0.5 * (1 / ie) * E.abs() ** 2).sum(0) + (0.5 * (1 / im) * H.abs() ** 2).sum(0)
            root = torch.sqrt(energy.sum())
            E = E / root
            H = H / root
        if full:
            eps_eff = torch.einsum("i,ijxyz,j->xyz", e, eps_t, e)
            mu_eff = torch.einsum("i,ijxyz,j->xyz", h, mu_t, h)
            H = H / torch.sqrt(mu_eff / eps_eff)
            for m in (ie, im):  # grid.py:781-861: tensor media must be isotropic here
                if _is9(m) and not (torch.allclose(m[0], m[4]) and torch.allclose(m[4], m[8]) and all(
                        torch.allclose(m[q], torch.zeros_like(m[q])) for q in (1, 2, 3, 5, 6, 7))):
                    raise NotImplementedError("Gaussian or planewave sources within anisotropic materials")
        else:
            H = H / torch.sqrt(ie / im)
        # calculate_time_offset_yee (fdtdx/core/grid.py:720-880), uniform edges
        edges = [torch.arange(gs[ax] + 1, dtype=dt_) * self.dx for ax in range(3)]
        cphys = torch.zeros(3, dtype=dt_)
        cphys[h_ax] = center[0] * self.dx
        cphys[v_ax] = center[1] * self.dx

        def pos(offsets):
            coords = []
            for ax in range(3):
                ed = edges[ax]
                coords.append(ed[:-1] if offsets[ax] == 0 else 0.5 * (ed[:-1] + ed[1:]))
            X, Y, Z = torch.meshgrid(*coords, indexing="ij")
            return torch.stack([X, Y, Z], -1) - cphys

        xyz_E = torch.stack([pos((0.5, 0, 0)), pos((0, 0.5, 0)), pos((0, 0, 0.5))])
        xyz_H = torch.stack([pos((0, 0.5, 0.5)), pos((0.5, 0, 0.5)), pos((0.5, 0.5, 0))])
        travel_E = -(xyz_E @ k)
        travel_H = -(xyz_H @ k)
        ie0 = ie[0]
        im0 = im[0] if isinstance(im, torch.Tensor) else im
        n_r = 1 / torch.sqrt(ie0 * im0)
        vel = (C0 / n_r)[None]
        return E, H, travel_E / (vel * self.dt), travel_H / (vel * self.dt)

    # ---- detectors
    def _setup_detector(self, d) -> ODetector:
        name = type(d).__name__
        on = d.on_list(_ConfigShim(self))
        idx, cnt = [-1] * self.T, 0
        for t in range(self.T):
            if on[t]:
                idx[t] = cnt
                cnt += 1
        if name in ("PhasorDetector", "PhasorPoyntingFluxDetector"):
            on_arr = np.asarray(on, np.float64)
            window = on_arr if d.apodization is None else d.apodization.get_window(np.arange(self.T) * self.dt) * on_arr
            wsum = float(window.sum())
            scale = 2 / wsum if d.scaling_mode == "continuous" else float(d.resolve_dft_stride(_ConfigShim(self)))
            return ODetector(d, "phasor", on, idx, window=window, scale=scale)
        kind = {"FieldDetector": "field", "PoyntingFluxDetector": "flux", "EnergyDetector": "energy"}[name]
        return ODetector(d, kind, on, idx)

    def pad(self, f: torch.Tensor) -> torch.Tensor:
        """pad_fields_for_boundaries (fdtdx/fdtd/update.py:92-136) without symmetry planes."""
        return pad_fields(f, self.periodic, self.bloch)

    # ---- state
    def init_state(self) -> "OState":
        fdt = self.field_dtype
        z = torch.zeros((3, *self.shape), dtype=fdt)
        psi_E = {p.name: (torch.zeros(_slab_shape(self.shape, p), dtype=fdt),) * 2 for p in self.pmls}
        psi_H = {p.name: (torch.zeros(_slab_shape(self.shape, p), dtype=fdt),) * 2 for p in self.pmls}
        det = {}
        for od in self.detectors:
            d = od.obj
            gs = d.grid_shape
            n_on = sum(od.on)
            if od.kind == "phasor":
                F, Cc = len(d.wave_characters), len(d.recorded_components)
                cdt = torch.complex128 if self.dtype == torch.float64 else torch.complex64
                shp = (1, F, Cc) if d.reduce_volume else (1, F, Cc, *gs)
                det[d.name] = {"phasor": torch.zeros(shp, dtype=cdt)}
            elif od.kind == "field":
                Cc = len(d.recorded_components)
                det[d.name] = {"fields": torch.zeros((n_on, Cc) if d.reduce_volume else (n_on, Cc, *gs), dtype=self.dtype)}
            elif od.kind == "flux":
                if d.keep_all_components:
                    shp = (n_on, 3) if d.reduce_volume else (n_on, 3, *gs)
                else:
                    shp = (n_on, 1) if d.reduce_volume else (n_on, *gs)
                det[d.name] = {"poynting_flux": torch.zeros(shp, dtype=self.dtype)}
            else:
                det[d.name] = {"energy": torch.zeros((n_on, 1) if d.reduce_volume else (n_on, *gs), dtype=self.dtype)}
        P = None
        if self.disp is not None:
            zp = torch.zeros((self.disp[0].shape[0], 3, *self.shape), dtype=fdt)
            P = (zp, zp.clone())
        return OState(0, z.clone(), z.clone(), psi_E, psi_H, det, [], P)


class _ConfigShim:
    """The few config attributes the objects' on-list helpers read."""

    def __init__(self, sc: OracleScene):
        self.time_steps_total = sc.T
        self.time_step_duration = sc.dt


def _slab_shape(shape, p: OPml):
    return tuple(b - a for a, b in (s.indices(n)[:2] for s, n in zip(p.grid_slice, shape)))


@dataclass
class OState:
    t: int
    E: torch.Tensor
    H: torch.Tensor
    psi_E: dict
    psi_H: dict
    det: dict
    rec: list = field(default_factory=list)
    P: tuple | None = None  # (P_curr, P_prev) of the dispersive poles, (poles, 3, *grid)


# --------------------------------------------------------------------------------------------
# sources
# --------------------------------------------------------------------------------------------


def _src_time(sc: OracleScene, s: OSource, t: float, eside: bool):
    """(is_on, time step used) per update.py:494-519 / 824-849 and source.py:41-49."""
    half = 0.0 if eside else 0.5
    if s.default_on:
        return True, t + half
    ti = int(t)
    on = s.on[jax_index(sc.T, ti)]
    adj = float(s.on_idx[ti]) if 0 <= ti < sc.T else 0.0
    return on, adj + half


def _is9(m) -> bool:
    return isinstance(m, torch.Tensor) and m.dim() > 0 and m.shape[0] == 9


def contract_orientation(inv_local, orient: torch.Tensor) -> torch.Tensor:
    """_contract_orientation (dipole.py:15-37): sum_j inv_ij p_j for a 9-component tensor,
    inv_i p_i for the isotropic / diagonal forms (a scalar or 1-component value broadcasts)."""
    if _is9(inv_local):
        return torch.einsum("ij...,j->i...", inv_local.reshape(3, 3, *inv_local.shape[1:]), orient.to(inv_local.dtype))
    return inv_local * orient.reshape(3, 1, 1, 1)


def _dipole_inject(F, o, s: OSource, scale, sign):
    """dipole.py:219-232 / 260-273: one component for an untilted dipole in an isotropic or
    diagonal medium, every component otherwise (tilted, or a full-tensor medium)."""
    oriented = contract_orientation(s.inv_local, s.orient)
    if o.azimuth_angle == 0.0 and o.elevation_angle == 0.0 and not _is9(s.inv_local):
        return _add_at(F, (o.polarization, *o.grid_slice), sign * (scale * oriented[o.polarization]))
    for axis in range(3):
        F = _add_at(F, (axis, *o.grid_slice), sign * (scale * oriented[axis]))
    return F


def _source_update_E(sc: OracleScene, s: OSource, E, inv_eps, t: float, inverse: bool):
    o = s.obj
    c = sc.courant
    dt_ = sc.dtype
    if s.kind == "dipole":
        if o.source_type != "electric":
            return E
        amp = profile_amplitude(o.temporal_profile, torch.tensor(t, dtype=dt_) * sc.dt,
                                o.wave_character.get_period(), o.wave_character.phase_shift)
        sign = -1.0 if not inverse else 1.0
        scale = c * o.amplitude * o.static_amplitude_factor * amp
        return _dipole_inject(E, o, s, scale, sign)
    # TFSF plane E-side (tfsf.py:193-308, 739-771)
    n = o.grid_shape.index(1)
    a_ax, b_ax = (n + 1) % 3, (n + 2) % 3
    sign = 1 if o.direction == "+" else -1
    if inverse:
        sign = -sign
    ies = inv_eps.detach()[(slice(None), *o.grid_slice)]
    amp = {}
    for ax in (a_ax, b_ax):
        if s.h_filter is not None:  # linear interpolation of the filtered profile, 0 outside (tfsf.py:256-261)
            idx = (t + s.off_H[ax]).to(torch.float64)
            xs = np.arange(len(s.h_filter), dtype=np.float64)
            vals = np.interp(idx.numpy().ravel(), xs, s.h_filter, left=0.0, right=0.0).reshape(tuple(idx.shape))
            amp[ax] = torch.from_numpy(vals).to(sc.dtype) * o.static_amplitude_factor
            continue
        time_H = (t + s.off_H[ax]) * sc.dt
        amp[ax] = profile_amplitude(o.temporal_profile, time_H, o.wave_character.get_period(),
                                    o.wave_character.phase_shift) * o.static_amplitude_factor
    if _is9(ies):  # fully anisotropic face (tfsf.py:287-299): every row picks up both tangential terms
        Hb_inc, Ha_inc = s.H_inc[b_ax] * amp[b_ax], s.H_inc[a_ax] * amp[a_ax]
        for row in (n, a_ax, b_ax):
            corr = c * (ies[row * 3 + a_ax] * Hb_inc + ies[row * 3 + b_ax] * (-Ha_inc))
            E = _add_at(E, (row, *o.grid_slice), sign * corr)
        return E
    Hb = s.H_inc[b_ax] * amp[b_ax] * c * ies[min(a_ax, ies.shape[0] - 1)]
    Ha = s.H_inc[a_ax] * amp[a_ax] * c * ies[min(b_ax, ies.shape[0] - 1)]
    E = _add_at(E, (a_ax, *o.grid_slice), sign * Hb)
    E = _add_at(E, (b_ax, *o.grid_slice), -sign * Ha)
    return E


def _source_update_H(sc: OracleScene, s: OSource, H, inv_mu, t: float, inverse: bool):
    o = s.obj
    c = sc.courant
    dt_ = sc.dtype
    if s.kind == "dipole":
        if o.source_type != "magnetic":
            return H
        amp = profile_amplitude(o.temporal_profile, torch.tensor(t, dtype=dt_) * sc.dt,
                                o.wave_character.get_period(), o.wave_character.phase_shift)
        sign = -1.0 if not inverse else 1.0
        scale = c * o.amplitude * o.static_amplitude_factor * amp
        return _dipole_inject(H, o, s, scale, sign)
    n = o.grid_shape.index(1)
    a_ax, b_ax = (n + 1) % 3, (n + 2) % 3
    sign = 1 if o.direction == "+" else -1
    if inverse:
        sign = -sign
    amp = {}
    for ax in (a_ax, b_ax):
        time_E = (t + s.off_E[ax]) * sc.dt
        amp[ax] = profile_amplitude(o.temporal_profile, time_E, o.wave_character.get_period(),
                                    o.wave_character.phase_shift) * o.static_amplitude_factor
    if _is9(inv_mu):  # fully anisotropic face (tfsf.py:384-393)
        ims = inv_mu.detach()[(slice(None), *o.grid_slice)]
        Ea_inc, Eb_inc = s.E_inc[a_ax] * amp[a_ax], s.E_inc[b_ax] * amp[b_ax]
        for row in (n, a_ax, b_ax):
            corr = c * (ims[row * 3 + a_ax] * (-Eb_inc) + ims[row * 3 + b_ax] * Ea_inc)
            H = _add_at(H, (row, *o.grid_slice), sign * corr)
        return H
    if isinstance(inv_mu, torch.Tensor):
        ims = inv_mu.detach()[(slice(None), *o.grid_slice)]
        im_a, im_b = ims[min(a_ax, ims.shape[0] - 1)], ims[min(b_ax, ims.shape[0] - 1)]
    else:
        im_a = im_b = inv_mu
    Ea = s.E_inc[a_ax] * amp[a_ax] * c * im_b
    Eb = s.E_inc[b_ax] * amp[b_ax] * c * im_a
    H = _add_at(H, (b_ax, *o.grid_slice), sign * Ea)
    H = _add_at(H, (a_ax, *o.grid_slice), -sign * Eb)
    return H


def _apply_sources(sc, field_, mat, t: int, eside: bool, inverse: bool):
    for s in sc.sources:
        on, tt = _src_time(sc, s, t, eside)
        if not on:
            continue
        if eside:
            field_ = _source_update_E(sc, s, field_, mat, tt, inverse)
        else:
            field_ = _source_update_H(sc, s, field_, mat, tt, inverse)
    return field_


def _walls(sc, F, walls):
    for b in walls:
        c1, c2 = ((1, 2), (0, 2), (0, 1))[b.axis]
        F = _set_at(F, (c1, *b.grid_slice), 0.0)
        F = _set_at(F, (c2, *b.grid_slice), 0.0)
    return F


# --------------------------------------------------------------------------------------------
# full 3x3 anisotropic branch (uniform grid)
# --------------------------------------------------------------------------------------------


def expand_to_3x3(arr):
    """fdtdx/core/misc.py:557-611: (1 | 3 | 9, *grid) or a scalar -> (3, 3, *grid)."""
    if arr is None:
        return None
    if not isinstance(arr, torch.Tensor) or arr.dim() == 0:
        a = torch.as_tensor(arr, dtype=torch.float64)
        return (torch.eye(3, dtype=a.dtype) * a)[:, :, None, None, None]
    n = arr.shape[0]
    if n == 9:
        return arr.reshape(3, 3, *arr.shape[1:])
    z = torch.zeros(arr.shape[1:], dtype=arr.dtype)
    d = [arr[0], arr[0], arr[0]] if n == 1 else [arr[0], arr[1], arr[2]]
    return torch.stack([torch.stack([d[r] if q == r else z for q in range(3)]) for r in range(3)])


def _tensor_inverse(m: torch.Tensor) -> torch.Tensor:
    """Per-cell inverse of a (3, 3, ...) tensor field (3 x 3 blocks moved last and back)."""
    k = m.dim() - 2
    perm = tuple(range(2, 2 + k)) + (0, 1)
    back = (k, k + 1) + tuple(range(k))
    return torch.linalg.inv(m.permute(perm)).permute(back)


def aniso_update_matrices(inv, sigma, c: float, eta_factor: float, reverse: bool = False):
    """fdtdx/fdtd/misc.py:69-129: A, B of E^(n+1) = A E^n + B curl (forward) or of the reverse
    update; M1 = I + (c eta / 2) inv sigma, M2 = I - (c eta / 2) inv sigma, forward A = M1^-1 M2,
    B = c M1^-1 inv, reverse A = M2^-1 M1, B = c M2^-1 inv."""
    grid = inv.shape[2:]
    eye = torch.eye(3, dtype=inv.dtype).reshape(3, 3, 1, 1, 1).expand(3, 3, *grid)
    M1, M2 = eye.clone(), eye.clone()
    if sigma is not None:
        f = c * eta_factor / 2 * torch.einsum("ijxyz,jkxyz->ikxyz", inv, sigma.expand(3, 3, *grid))
        M1 = M1 + f
        M2 = M2 - f
    to_last = (2, 3, 4, 0, 1)
    back = (3, 4, 0, 1, 2)
    lhs, rhs = (M2, M1) if reverse else (M1, M2)
    A = torch.linalg.solve(lhs.permute(to_last), rhs.permute(to_last)).permute(back)
    B = c * torch.linalg.solve(lhs.permute(to_last), inv.expand(3, 3, *grid).permute(to_last)).permute(back)
    return A, B


def avg_aniso_E(field_pad, component: int, location: int):
    """fdtdx/fdtd/misc.py:132-171 (uniform grid): component `component` of a padded E-type field
    averaged onto the Yee location of `location`."""
    s = field_pad[component]
    la, ca = location, component
    out = (s + torch.roll(s, -1, dims=la) + torch.roll(s, 1, dims=ca)
           + torch.roll(torch.roll(s, -1, dims=la), 1, dims=ca)) / 4
    return out[1:-1, 1:-1, 1:-1]


def avg_aniso_H(field_pad, component: int, location: int):
    """fdtdx/fdtd/misc.py:174-213 (uniform grid), the H-type stencil."""
    s = field_pad[component]
    la, ca = location, component
    out = (s + torch.roll(s, 1, dims=la) + torch.roll(s, -1, dims=ca)
           + torch.roll(torch.roll(s, 1, dims=la), -1, dims=ca)) / 4
    return out[1:-1, 1:-1, 1:-1]


def aniso_apply(A, B, F, curl, pad, avg, sign: float):
    """Rows of update.py:474-492 / 791-807: F_i = sum_j A_ij F_j@i + sign sum_j B_ij curl_j@i,
    the diagonal terms local, the off-diagonal ones averaged onto component i's location
    (``pad`` is the scene's halo, Bloch phases included)."""
    F_pad, K_pad = pad(F), pad(curl)
    rows = []
    for i in range(3):
        acc_a = A[i, i] * F[i]
        acc_b = B[i, i] * curl[i]
        for j in range(3):
            if j == i:
                continue
            acc_a = acc_a + A[i, j] * avg(F_pad, j, i)
            acc_b = acc_b + B[i, j] * avg(K_pad, j, i)
        rows.append(acc_a + sign * acc_b)
    return torch.stack(rows)


def _full_tensor(inv, sigma) -> bool:
    return (isinstance(inv, torch.Tensor) and inv.dim() > 0 and inv.shape[0] == 9) or (
        sigma is not None and sigma.shape[0] == 9)


# --------------------------------------------------------------------------------------------
# updates
# --------------------------------------------------------------------------------------------


def update_E(sc: OracleScene, t: int, E, H, psi_E, inv_eps, simulate_boundaries=True, P=None):
    """fdtdx/fdtd/update.py:256-523 (isotropic / diagonal branch).  With dispersive poles and
    their polarisation ``P`` = (P_curr, P_prev) given, the ADE correction of update.py:316-350
    is applied and (E, psi_E, P_new) returned."""
    c = sc.courant
    E_old = E
    curl, psi_E = curl_H(sc.pad(H), psi_E, sc.pmls, simulate_boundaries)
    sig = sc.sigma_E
    if _full_tensor(inv_eps, sig):  # update.py:356-492
        if P is not None:
            raise NotImplementedError("dispersion with full-tensor materials")
        A, B = aniso_update_matrices(expand_to_3x3(inv_eps), expand_to_3x3(sig), c, ETA0)
        E = aniso_apply(A, B, E, curl, sc.pad, avg_aniso_E, 1.0)
        E = _apply_sources(sc, E, inv_eps, t, True, False)
        return _walls(sc, E, sc.pec), psi_E
    factor = 1
    if sig is not None:
        factor = 1 - c * sig * ETA0 * inv_eps / 2
    E = factor * E + c * curl * inv_eps
    if P is not None:
        # P_hat = c1 P^n + c2 P^{n-1} + c3 E^n;  E += inv_eps sum_poles (P^n - P_hat)
        c1, c2, c3 = sc.disp
        P_curr, P_prev = P
        P_hat = c1 * P_curr + c2 * P_prev + c3 * E_old
        E = E + inv_eps * (P_curr - P_hat).sum(0)
        P = (P_hat, P_curr)
    if sig is not None:
        E = E / (1 + c * sig * ETA0 * inv_eps / 2)
    E = _apply_sources(sc, E, inv_eps, t, True, False)
    if P is not None:
        return _walls(sc, E, sc.pec), psi_E, P
    return _walls(sc, E, sc.pec), psi_E


def update_H(sc: OracleScene, t: int, E, H, psi_H, inv_mu, simulate_boundaries=True):
    """fdtdx/fdtd/update.py:689-853 (isotropic / diagonal branch)."""
    c = sc.courant
    curl, psi_H = curl_E(sc.pad(E), psi_H, sc.pmls, simulate_boundaries)
    sig = sc.sigma_H
    if _full_tensor(inv_mu, sig):  # update.py:751-807
        A, B = aniso_update_matrices(expand_to_3x3(inv_mu), expand_to_3x3(sig), c, 1 / ETA0)
        H = aniso_apply(A, B, H, curl, sc.pad, avg_aniso_H, -1.0)
        H = _apply_sources(sc, H, inv_mu, t, False, False)
        return _walls(sc, H, sc.pmc), psi_H
    factor = 1
    if sig is not None:
        factor = 1 - c * sig / ETA0 * inv_mu / 2
    H = factor * H - c * curl * inv_mu
    if sig is not None:
        H = H / (1 + c * sig / ETA0 * inv_mu / 2)
    H = _apply_sources(sc, H, inv_mu, t, False, False)
    return _walls(sc, H, sc.pmc), psi_H


def update_E_reverse(sc: OracleScene, t: int, E, H, psi_E, inv_eps):
    """fdtdx/fdtd/update.py:526-686."""
    c = sc.courant
    E = _apply_sources(sc, E, inv_eps, t, True, True)
    curl, _ = curl_H(sc.pad(H), psi_E, sc.pmls, False)
    sig = sc.sigma_E
    if _full_tensor(inv_eps, sig):  # update.py:641-676
        A, B = aniso_update_matrices(expand_to_3x3(inv_eps), expand_to_3x3(sig), c, ETA0, reverse=True)
        return _walls(sc, aniso_apply(A, B, E, curl, sc.pad, avg_aniso_E, -1.0), sc.pec)
    factor = 1
    if sig is not None:
        E = E * (1 + c * sig * ETA0 * inv_eps / 2)
        factor = 1 - c * sig * ETA0 * inv_eps / 2
    E = (E - c * curl * inv_eps) / factor
    return _walls(sc, E, sc.pec)


def update_H_reverse(sc: OracleScene, t: int, E, H, psi_H, inv_mu):
    """fdtdx/fdtd/update.py:856-1007."""
    c = sc.courant
    H = _apply_sources(sc, H, inv_mu, t, False, True)
    curl, _ = curl_E(sc.pad(E), psi_H, sc.pmls, False)
    sig = sc.sigma_H
    if _full_tensor(inv_mu, sig):  # update.py:956-995
        A, B = aniso_update_matrices(expand_to_3x3(inv_mu), expand_to_3x3(sig), c, 1 / ETA0, reverse=True)
        return _walls(sc, aniso_apply(A, B, H, curl, sc.pad, avg_aniso_H, 1.0), sc.pmc)
    factor = 1
    if sig is not None:
        H = H * (1 + c * sig / ETA0 * inv_mu / 2)
        factor = 1 - c * sig / ETA0 * inv_mu / 2
    H = (H + c * curl * inv_mu) / factor
    return _walls(sc, H, sc.pmc)


# --------------------------------------------------------------------------------------------
# detectors and interfaces
# --------------------------------------------------------------------------------------------


def update_detectors(sc: OracleScene, t: int, E, H, H_prev, det: dict, inv_eps, inv_mu) -> dict:
    """fdtdx/fdtd/update.py:1040-1137 with each detector's update()."""
    out = dict(det)
    full = None
    for od in sc.detectors:
        d = od.obj
        if not od.on[jax_index(sc.T, t)]:
            continue
        gs = (slice(None), *d.grid_slice)
        if d.exact_interpolation:
            if full is None:
                full = interpolate_fields(sc.pad(E), sc.pad((H_prev + H) / 2))
            Er, Hr = full[0][gs], full[1][gs]
        else:
            Er, Hr = E[gs], H[gs]
        st = det[d.name]
        if od.kind in ("phasor", "field"):
            EH = torch.stack([torch.cat([Er, Hr], 0)[COMPONENTS.index(cn)] for cn in d.recorded_components], 0)
        if od.kind == "phasor":
            time_passed = torch.tensor(float(t), dtype=sc.dtype) * sc.dt
            omegas = torch.tensor([2 * math.pi * wc.get_frequency() for wc in d.wave_characters], dtype=sc.dtype)
            ph = torch.exp(1j * (omegas * time_passed))
            ph = ph.reshape((len(omegas),) + (1,) * EH.ndim)
            w = float(od.window[jax_index(sc.T, t)])
            new = EH * ph * od.scale * w
            if d.reduce_volume:
                new = new.mean(dim=tuple(range(2, new.ndim)))
            res = st["phasor"] - new[None] if d.inverse else st["phasor"] + new[None]
            out[d.name] = {"phasor": res}
        elif od.kind == "field":
            if d.reduce_volume:
                EH = EH.mean(dim=(1, 2, 3))
            if EH.is_complex() and not st["fields"].is_complex():
                EH = EH.real  # a real state keeps the real part (JAX's complex -> float cast)
            idx = od.arr_idx[jax_index(sc.T, t)]
            out[d.name] = {"fields": _set_at(st["fields"], idx, EH)}
        elif od.kind == "flux":
            Hc = Hr.conj() if Hr.is_complex() else Hr  # Re(E x conj(H)) (core/physics/metrics.py:99-117)
            S = torch.stack([
                Er[1] * Hc[2] - Er[2] * Hc[1],
                Er[2] * Hc[0] - Er[0] * Hc[2],
                Er[0] * Hc[1] - Er[1] * Hc[0],
            ], 0)
            if S.is_complex():
                S = S.real
            pf = S if d.keep_all_components else S[d.propagation_axis]
            if d.direction == "-":
                pf = -pf
            if d.reduce_volume:
                pf = pf * (sc.dx * sc.dx)
                pf = pf.sum(dim=(1, 2, 3)) if d.keep_all_components else pf.sum().reshape(1)
            idx = od.arr_idx[jax_index(sc.T, t)]
            out[d.name] = {"poynting_flux": _set_at(st["poynting_flux"], idx, pf)}
        else:  # energy
            ie = inv_eps[gs]
            im = inv_mu[gs] if isinstance(inv_mu, torch.Tensor) else inv_mu
            if _is9(ie) or _is9(im):  # 0.5 Re(E* eps E) + 0.5 Re(H* mu H) (core/physics/metrics.py:34-51)
                eps_t = _tensor_inverse(expand_to_3x3(ie)).to(sc.dtype).expand(3, 3, *Er.shape[1:])
                mu_t = _tensor_inverse(expand_to_3x3(im)).to(sc.dtype).expand(3, 3, *Er.shape[1:])
                e = 0.5 * torch.einsum("ixyz,ijxyz,jxyz->xyz", Er.conj(), eps_t.to(Er.dtype), Er).real \
                    + 0.5 * torch.einsum("ixyz,ijxyz,jxyz->xyz", Hr.conj(), mu_t.to(Hr.dtype), Hr).real
            elif Er.is_complex():  # |E|^2 (core/physics/metrics.py:15-60)
                e = (0.5 * (1 / ie) * Er.abs() ** 2).sum(0) + (0.5 * (1 / im) * Hr.abs() ** 2).sum(0)
            else:
                e = (0.5 * (1 / ie) * Er**2).sum(0) + (0.5 * (1 / im) * Hr**2).sum(0)
            if d.reduce_volume:
                e = (e * sc.dx**3).sum().reshape(1)
            idx = od.arr_idx[jax_index(sc.T, t)]
            out[d.name] = {"energy": _set_at(st["energy"], idx, e)}
    return out


def interface_slice(p: OPml, shape):
    st = [s.indices(n)[:2] for s, n in zip(p.grid_slice, shape)]
    lo, hi = st[p.axis]
    st[p.axis] = (lo, lo + 1) if p.direction == "+" else (hi - 1, hi)
    return tuple(slice(a, b) for a, b in st)


def collect_interfaces(sc: OracleScene, E, H) -> dict:
    """fdtdx/fdtd/misc.py:10-35."""
    return {f"{p.name}_{fs}": F[(slice(None), *interface_slice(p, sc.shape))].clone()
            for fs, F in (("E", E), ("H", H)) for p in sc.pmls}


def add_interfaces(sc: OracleScene, E, H, values: dict):
    """fdtdx/fdtd/misc.py:38-66."""
    for p in sc.pmls:
        sl = (slice(None), *interface_slice(p, sc.shape))
        E = _set_at(E, sl, values[f"{p.name}_E"])
        H = _set_at(H, sl, values[f"{p.name}_H"])
    return E, H


# --------------------------------------------------------------------------------------------
# steps and runs
# --------------------------------------------------------------------------------------------


def forward(sc: OracleScene, st: OState, inv_eps=None, inv_mu=None, record_detectors=True,
            record_boundaries=False, simulate_boundaries=True) -> OState:
    """One forward step, fdtdx/fdtd/forward.py:83-156."""
    inv_eps = sc.inv_eps if inv_eps is None else inv_eps
    inv_mu = sc.inv_mu if inv_mu is None else inv_mu
    t = st.t
    H_prev = st.H
    P = st.P
    if sc.disp is not None:
        E, psi_E, P = update_E(sc, t, st.E, st.H, st.psi_E, inv_eps, simulate_boundaries, P=st.P)
    else:
        E, psi_E = update_E(sc, t, st.E, st.H, st.psi_E, inv_eps, simulate_boundaries)
    H, psi_H = update_H(sc, t, E, st.H, st.psi_H, inv_mu, simulate_boundaries)
    rec = st.rec
    if record_boundaries and sc.records(t):
        rec = rec + [collect_interfaces(sc, E, H)]
    det = update_detectors(sc, t, E, H, H_prev, st.det, inv_eps, inv_mu) if record_detectors else st.det
    return OState(t + 1, E, H, psi_E, psi_H, det, rec, P)


def backward(sc: OracleScene, st: OState) -> OState:
    """One reverse step with reset_fields=False and no detectors (fdtdx/fdtd/backward.py:62-135)."""
    if sc.disp is not None:  # fdtd/initialization.py:674-685: the ADE recurrence is not reversed
        raise NotImplementedError("dispersive materials have no time-reversed step")
    t = st.t - 1
    E, H = st.E, st.H
    if st.rec:
        E, H = add_interfaces(sc, E, H, sc.recorded(st.rec, t))
    H = update_H_reverse(sc, t, E, H, st.psi_H, sc.inv_mu)
    E = update_E_reverse(sc, t, E, H, st.psi_E, sc.inv_eps)
    return OState(t, E, H, st.psi_E, st.psi_H, st.det, st.rec)


def run(sc: OracleScene, n_steps: int | None = None, record_boundaries=False, state: OState | None = None) -> OState:
    st = sc.init_state() if state is None else state
    n = sc.T if n_steps is None else n_steps
    with torch.no_grad():
        for _ in range(n):
            st = forward(sc, st, record_boundaries=record_boundaries)
    return st


def reversible_gradient(sc: OracleScene, final: OState, cot_det: dict, cot_E=None, cot_H=None, with_mu=False):
    """d loss / d inv_eps by the reference's custom VJP (fdtdx/fdtd/fdtd.py:215-333).

    Reverse-reconstructs the state step by step (psi frozen, interfaces re-imposed) and
    applies the VJP of one forward step at each reconstructed state, from t = T-1 down to
    t = -1 (the reference's loop condition ``time_step >= 0`` admits one step at t = -1).
    Cotangents follow torch's convention for complex detector states.  With ``with_mu``
    (an inv_mu array) returns ``(d/d inv_eps, d/d inv_mu)``, the reference's cot[5] and
    cot[6] (fdtd.py:330-331).
    """
    zE = torch.zeros_like(final.E)
    lam = {
        "E": zE.clone() if cot_E is None else cot_E.clone(),
        "H": zE.clone() if cot_H is None else cot_H.clone(),
        "psi_E": {k: (torch.zeros_like(a), torch.zeros_like(b)) for k, (a, b) in final.psi_E.items()},
        "psi_H": {k: (torch.zeros_like(a), torch.zeros_like(b)) for k, (a, b) in final.psi_H.items()},
        "det": {k: {k2: cot_det.get(k, {}).get(k2, torch.zeros_like(v2)) for k2, v2 in v.items()}
                for k, v in final.det.items()},
    }
    grad = torch.zeros_like(sc.inv_eps)
    if with_mu and not isinstance(sc.inv_mu, torch.Tensor):
        raise ValueError("with_mu needs an inv_mu array")
    grad_mu = torch.zeros_like(sc.inv_mu) if with_mu else None
    st = final
    while st.t >= 0:
        st = backward(sc, st)
        E = st.E.clone().requires_grad_(True)
        H = st.H.clone().requires_grad_(True)
        pE = {k: (a.clone().requires_grad_(True), b.clone().requires_grad_(True)) for k, (a, b) in st.psi_E.items()}
        pH = {k: (a.clone().requires_grad_(True), b.clone().requires_grad_(True)) for k, (a, b) in st.psi_H.items()}
        det_in = {k: {k2: v2.clone().requires_grad_(True) for k2, v2 in v.items()} for k, v in st.det.items()}
        ie = sc.inv_eps.clone().requires_grad_(True)
        im = sc.inv_mu.clone().requires_grad_(True) if with_mu else None
        out = forward(sc, OState(st.t, E, H, pE, pH, det_in, []), inv_eps=ie, inv_mu=im, record_detectors=True)
        outs, cots, ins = [out.E, out.H], [lam["E"], lam["H"]], [E, H, ie]
        for k in pE:
            outs += [out.psi_E[k][0], out.psi_E[k][1], out.psi_H[k][0], out.psi_H[k][1]]
            cots += [lam["psi_E"][k][0], lam["psi_E"][k][1], lam["psi_H"][k][0], lam["psi_H"][k][1]]
            ins += [pE[k][0], pE[k][1], pH[k][0], pH[k][1]]
        dkeys = [(k, k2) for k, v in det_in.items() for k2 in v]
        for k, k2 in dkeys:
            outs.append(out.det[k][k2])
            cots.append(lam["det"][k][k2])
            ins.append(det_in[k][k2])
        if with_mu:
            ins.append(im)
        pairs = [(o, c) for o, c in zip(outs, cots) if o.requires_grad]
        g = torch.autograd.grad([o for o, _ in pairs], ins, grad_outputs=[c for _, c in pairs], allow_unused=True)
        g = [torch.zeros_like(x) if gi is None else gi for gi, x in zip(g, ins)]
        lam["E"], lam["H"] = g[0], g[1]
        grad = grad + g[2]
        q = 3
        for k in pE:
            lam["psi_E"][k] = (g[q], g[q + 1])
            lam["psi_H"][k] = (g[q + 2], g[q + 3])
            q += 4
        for k, k2 in dkeys:
            lam["det"][k][k2] = g[q]
            q += 1
        if with_mu:
            grad_mu = grad_mu + g[q]
    return (grad, grad_mu) if with_mu else grad


def autograd_gradient(sc: OracleScene, loss_fn, n_steps: int | None = None, wrt: str = "eps") -> torch.Tensor:
    """Exact gradient of loss_fn(final detector states) by autograd through the whole forward run
    with respect to inv_eps (``wrt="eps"``) or the inv_mu array (``wrt="mu"``)."""
    x = (sc.inv_eps if wrt == "eps" else sc.inv_mu).clone().requires_grad_(True)
    st = sc.init_state()
    n = sc.T if n_steps is None else n_steps
    for _ in range(n):
        st = forward(sc, st, inv_eps=x) if wrt == "eps" else forward(sc, st, inv_mu=x)
    loss = loss_fn(st.det)
    (g,) = torch.autograd.grad(loss, [x])
    return g
