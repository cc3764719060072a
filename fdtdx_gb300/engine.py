"""Host setup of the native plan: scene -> ``FdtdDesc`` tables, plan lifecycle, calls.

Everything computed here is per-simulation setup that the reference does once in
``place_on_grid`` / ``apply`` of each object or in the per-step Python of its
update functions; the kernels receive it as small device tables:

* CPML coefficient vectors (perfectly_matched_layer.py:97-136, 231-275)
* per-step source tables: on/off, on/off-adjusted time step, and the carrier
  phase reduced mod 2 pi in float64 (source.py:41-66, profile.py:253-345)
* TFSF incident profiles and Yee time offsets of a plane source
  (linear_polarization.py:168-358, tfsf.py:144-190, fdtdx/core/grid.py:720-880)
* per-step detector tables: state slot, and the complex DFT weight
  exp(i w t dt) * scale * window[t] of phasor detectors (phasor.py:118-235)

Table index ``t + 1`` holds time step ``t`` for t in [-1, T]; the reference indexes its
per-step arrays with JAX semantics, so step -1 reads the last entry and step T
(clamped) reads it too.
"""

from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from fdtdx_gb300 import _native as N
from fdtdx_gb300 import constants
from fdtdx_gb300.config import SimulationConfig
from fdtdx_gb300.container import ArrayContainer, ObjectContainer
from fdtdx_gb300.core import GaussianPulseProfile, SingleFrequencyProfile
from fdtdx_gb300.objects import (
    COMPONENTS,
    EnergyDetector,
    FieldDetector,
    LinearlyPolarizedPlaneSource,
    PerfectElectricConductor,
    PerfectlyMatchedLayer,
    PerfectMagneticConductor,
    PeriodicBoundary,
    PhasorDetector,
    PointDipoleSource,
    PoyntingFluxDetector,
)

TWO_PI = 2.0 * math.pi


def _jax_index(t: int, n: int) -> int:
    """Index a length-n array at t the way a JAX gather does (negative wraps once, overflow clamps)."""
    if t < 0:
        t += n
    return min(max(t, 0), n - 1)


@dataclass
class SourceTables:
    desc: N.SourceDesc
    keep: list = field(default_factory=list)  # numpy arrays referenced by desc


def _profile_params(profile, wave, dt: float) -> tuple[int, float, float, float, float, float]:
    """(kind, omega [rad/s], phase0, ramp_inv_steps, t0_steps, inv_two_sigma2) of a temporal profile."""
    if isinstance(profile, SingleFrequencyProfile):
        period = wave.get_period()
        omega = TWO_PI / period
        phase0 = wave.phase_shift + profile.phase_shift
        ramp_inv = dt / (profile.num_startup_periods * period)
        return N.PROFILE_CW, omega, phase0, ramp_inv, 0.0, 0.0
    if isinstance(profile, GaussianPulseProfile):
        omega = TWO_PI * profile.center_wave.get_frequency()
        phase0 = wave.phase_shift + profile.center_wave.phase_shift
        sigma = profile.sigma_t
        return N.PROFILE_GAUSSIAN, omega, phase0, 0.0, 6.0 * sigma / dt, dt * dt / (2.0 * sigma * sigma)
    raise NotImplementedError(f"temporal profile {type(profile).__name__} is not supported")


def source_time_tables(src, config: SimulationConfig) -> tuple[np.ndarray, np.ndarray]:
    """(on, teff) for t in [-1, T]: the on/off state and the on/off-adjusted time step."""
    T = config.time_steps_total
    ts = np.arange(-1, T + 1)
    if src.switch.is_default_always_on:
        return np.ones(T + 2, np.uint8), ts.astype(np.float64)
    on_list = src.switch.calculate_on_list(T, config.time_step_duration)
    idx = src.switch.calculate_time_step_to_on_arr_idx(T, config.time_step_duration)
    on = np.array([on_list[_jax_index(t, T)] for t in ts], np.uint8)
    # linear_interpolated_indexing at an integer point: the entry, or 0 outside the array
    teff = np.array([float(idx[t]) if 0 <= t < T else 0.0 for t in ts], np.float64)
    return on, teff


def build_source(src, arrays: ArrayContainer, config: SimulationConfig) -> list[SourceTables]:
    """The source records of one source object: one per plane source, one per injected
    component of a point dipole."""
    dt = config.time_step_duration
    c = config.courant_number
    kind, omega, phase0, ramp_inv, t0s, inv2s2 = _profile_params(src.temporal_profile, src.wave_character, dt)
    on, teff = source_time_tables(src, config)
    ph_E = np.mod(omega * dt * teff + phase0, TWO_PI).astype(np.float32)
    ph_H = np.mod(omega * dt * (teff + 0.5) + phase0, TWO_PI).astype(np.float32)
    d = N.SourceDesc()
    st = src.grid_slice_tuple
    for a in range(3):
        d.lo[a], d.hi[a] = st[a]
    d.profile = kind
    d.omega_dt = omega * dt
    d.ramp_inv_steps = ramp_inv
    d.t0_steps = t0s
    d.inv_two_sigma2 = inv2s2
    keep = [ph_E, ph_H, teff.astype(np.float32), on]
    d.phase_E = ph_E.ctypes.data
    d.phase_H = ph_H.ctypes.data
    d.teff = keep[2].ctypes.data
    d.on = on.ctypes.data
    if isinstance(src, PointDipoleSource):
        if src.grid_shape != (1, 1, 1):
            raise ValueError("a point dipole occupies exactly one cell")
        i, j, k = (st[0][0], st[1][0], st[2][0])
        magnetic = src.source_type == "magnetic"
        m = arrays.inv_permeabilities if magnetic else arrays.inv_permittivities
        # one record per injected component: the polarization axis alone for an axis-aligned
        # dipole, every axis the tilted orientation reaches otherwise (dipole.py:219-232), each
        # scaled by c * amplitude * inv_material[axis] * orientation[axis]
        orient = src.orientation
        full = isinstance(m, torch.Tensor) and m.dim() > 0 and m.shape[0] == 9
        if full:
            # a full tensor couples the orientation into every component: sum_j inv_aj p_j
            # (_contract_orientation, dipole.py:15-37); every component is injected
            t = m[:, i, j, k].detach().double().cpu().numpy().reshape(3, 3)
            oriented = t @ np.asarray(orient, dtype=np.float64)
            axes = [a for a in range(3) if oriented[a] != 0.0]
        else:
            axes = [src.polarization] if not src.is_tilted else [a for a in range(3) if orient[a] != 0.0]
        out = []
        for a in axes:
            if full:
                weight = float(oriented[a])
            else:
                if not isinstance(m, torch.Tensor):
                    local = float(m)
                else:
                    loc = m[:, i, j, k].detach().double().cpu().numpy()
                    if not magnetic and arrays.dispersive_c1 is not None:
                        # the medium at the carrier in dispersive scenes (dipole.py:168-180)
                        loc = _carrier_inv_eps(loc.reshape(-1, 1, 1, 1), arrays,
                                               (slice(i, i + 1), slice(j, j + 1), slice(k, k + 1)),
                                               src, config).reshape(-1)
                    local = float(loc[min(a, loc.shape[0] - 1)])
                weight = local * (1.0 if not src.is_tilted else orient[a])
            da = N.SourceDesc.from_buffer_copy(d)
            da.kind = N.SRC_DIPOLE
            da.component = a
            da.magnetic = 1 if magnetic else 0
            da.coef = c * src.amplitude * src.static_amplitude_factor * weight
            out.append(SourceTables(da, keep))
        return out
    if isinstance(src, LinearlyPolarizedPlaneSource):
        d.kind = N.SRC_PLANE
        d.normal_axis = src.propagation_axis
        d.sign = 1.0 if src.direction == "+" else -1.0
        d.coef = c * src.static_amplitude_factor
        incE, incH, offE, offH = plane_source_profiles(src, arrays, config)
        keep += [incE, incH, offE, offH]
        d.inc_E, d.inc_H, d.off_E, d.off_H = (x.ctypes.data for x in (incE, incH, offE, offH))
        if arrays.dispersive_c1 is not None:
            # dispersive scenes inject the E side with the broadband impedance-corrected profile,
            # read at the fractional time by linear interpolation (tfsf.py:21-141, 256-261)
            tab = np.ascontiguousarray(_plane_e_table(src, arrays, config), dtype=np.float32)
            keep.append(tab)
            d.e_table, d.n_e_table = tab.ctypes.data, int(tab.shape[0])
        return [SourceTables(d, keep)]
    raise NotImplementedError(f"source type {type(src).__name__} is not supported")


def _carrier_inv_eps(inv_slice: np.ndarray, arrays: ArrayContainer, sl, src, config: SimulationConfig) -> np.ndarray:
    """inv_eps of a slice as a source sees it in a dispersive scene: 1 / (eps_inf + Re chi) at
    the source's carrier (effective_inv_permittivity, fdtdx/dispersion.py:1254-1307)."""
    from fdtdx_gb300.dispersion import effective_inv_permittivity

    cs = [c[(slice(None), slice(None), *sl)].detach().double().cpu().numpy()
          for c in (arrays.dispersive_c1, arrays.dispersive_c2, arrays.dispersive_c3)]
    omega = 2 * math.pi * src.wave_character.get_frequency()
    return effective_inv_permittivity(inv_slice, cs[0], cs[1], cs[2], omega, config.time_step_duration)


def _plane_e_table(src, arrays: ArrayContainer, config: SimulationConfig) -> np.ndarray:
    """The E side's profile of a plane source in a dispersive scene at steps 0 .. T - 1: the raw
    profile filtered by sqrt(eps(omega) / eps(omega_c)) averaged over the source's cells
    (_build_dispersive_H_filter, fdtdx/objects/sources/tfsf.py:21-141)."""
    from fdtdx_gb300.dispersion import dispersive_h_filter

    T, dt = config.time_steps_total, config.time_step_duration
    raw = np.asarray(src.temporal_profile.get_amplitude(np.arange(T, dtype=np.float64) * dt,
                                                         src.wave_character.get_period(),
                                                         src.wave_character.phase_shift), dtype=np.float64)
    sl = (slice(None), slice(None), *src.grid_slice)
    cs = [c[sl].detach().double().cpu().numpy() for c in (arrays.dispersive_c1, arrays.dispersive_c2,
                                                          arrays.dispersive_c3)]
    inv_inf = arrays.inv_permittivities[(slice(None), *src.grid_slice)].detach().double().cpu().numpy()
    return dispersive_h_filter(raw, cs[0], cs[1], cs[2], inv_inf, 2 * math.pi * src.wave_character.get_frequency(), dt)


def _tensor3(m, face_shape) -> np.ndarray:
    """(3, 3, *face) tensor of a (1 | 3 | 9, *face) material slice or a scalar."""
    if not isinstance(m, np.ndarray):
        return np.broadcast_to(np.eye(3)[:, :, None, None, None] * m, (3, 3, *face_shape))
    if m.shape[0] == 9:
        return m.reshape(3, 3, *m.shape[1:])
    out = np.zeros((3, 3, *m.shape[1:]))
    for q in range(3):
        out[q, q] = m[min(q, m.shape[0] - 1)]
    return out


def _is_full(m) -> bool:
    return isinstance(m, np.ndarray) and m.shape[0] == 9


def _medium_scaling(src, ie, im, E, Hf, e_pol, h_pol):
    """Energy normalisation and impedance scaling of the incident profiles
    (linear_polarization.py:186-211).  In tensor media eps and mu are the per-cell inverses of
    the stored inverse tensors: the energy is 0.5 E.eps.E + 0.5 H.mu.H (metrics.py:34-51) and H
    is divided by sqrt(mu_eff / eps_eff) with eps_eff = e.eps.e, mu_eff = h.mu.h
    (tfsf.py:144-190); the plane must then lie in an isotropic tensor, as the reference's time
    offsets require (fdtdx/core/grid.py:781-861)."""
    if not (_is_full(ie) or _is_full(im)):
        if src.normalize_by_energy:
            energy = (0.5 * (1.0 / ie) * E**2).sum(axis=0) + (0.5 * (1.0 / im) * Hf**2).sum(axis=0)
            root = math.sqrt(float(energy.sum()))
            E = E / root
            Hf = Hf / root
        return E, Hf / np.sqrt(ie / im)
    face = E.shape[1:]
    inv_t = [_tensor3(m, face) for m in (ie, im)]
    eps_t, mu_t = (np.moveaxis(np.linalg.inv(np.moveaxis(t, (0, 1), (-2, -1))), (-2, -1), (0, 1)) for t in inv_t)
    if src.normalize_by_energy:
        energy = 0.5 * np.einsum("ixyz,ijxyz,jxyz->xyz", E, eps_t, E) + 0.5 * np.einsum("ixyz,ijxyz,jxyz->xyz", Hf, mu_t, Hf)
        root = math.sqrt(float(energy.sum()))
        E = E / root
        Hf = Hf / root
    eps_eff = np.einsum("i,ijxyz,j->xyz", np.asarray(e_pol, np.float64), eps_t, np.asarray(e_pol, np.float64))
    mu_eff = np.einsum("i,ijxyz,j->xyz", np.asarray(h_pol, np.float64), mu_t, np.asarray(h_pol, np.float64))
    Hf = Hf / np.sqrt(mu_eff / eps_eff)
    for m in (ie, im):
        if _is_full(m):
            if not (np.allclose(m[[1, 2, 3, 5, 6, 7]], 0.0) and np.allclose(m[0], m[4]) and np.allclose(m[4], m[8])):
                raise NotImplementedError("Gaussian or planewave sources within anisotropic materials")
    return E, Hf


def plane_source_profiles(src: LinearlyPolarizedPlaneSource, arrays: ArrayContainer, config: SimulationConfig):
    """Incident E/H profiles and Yee time offsets of an untilted plane source, each (3, face cells).

    Restates LinearlyPolarizedPlaneSource.apply (linear_polarization.py:168-358) for normal
    incidence on a uniform grid: profile -> E = a e_pol, H = a h_pol -> energy normalisation ->
    H / sqrt(inv_eps / inv_mu) -> offsets = -(k . r) n / (c dt) with r the Yee position of
    each component relative to the plane (calculate_time_offset_yee, fdtdx/core/grid.py:720-880).
    """
    if src.is_tilted:
        return _tilted_plane_profiles(src, arrays, config)
    n = src.propagation_axis
    h_ax, v_ax = src.horizontal_axis, src.vertical_axis
    shape = src.grid_shape
    prof_hv = src.amplitude_raw_hv(config.uniform_spacing())
    prof = prof_hv.T if h_ax > v_ax else prof_hv
    amp = np.expand_dims(prof, axis=n)  # grid-shaped (face in x, y, z order)
    e_pol, h_pol, k = src.polarization_vectors()
    E = amp[None] * e_pol[:, None, None, None]
    Hf = amp[None] * h_pol[:, None, None, None]
    sl = (slice(None), *src.grid_slice)
    ie = arrays.inv_permittivities[sl].detach().double().cpu().numpy()
    if arrays.dispersive_c1 is not None:  # impedance, energy and offsets at the carrier (linear_polarization.py:186-211)
        ie = _carrier_inv_eps(ie, arrays, src.grid_slice, src, config)
    mu = arrays.inv_permeabilities
    im = mu[sl].detach().double().cpu().numpy() if isinstance(mu, torch.Tensor) else float(mu)
    E, Hf = _medium_scaling(src, ie, im, E, Hf, e_pol, h_pol)
    # Yee positions along the normal: 0.5 dx for components staggered along it
    stag_E = [0.5 if comp == n else 0.0 for comp in range(3)]
    stag_H = [0.0 if comp == n else 0.5 for comp in range(3)]
    dx, dt = config.uniform_spacing(), config.time_step_duration
    ie0 = ie[0]
    im0 = im[0] if isinstance(im, np.ndarray) else im
    n_r = 1.0 / np.sqrt(ie0 * im0)
    scale = n_r / (constants.c * dt)
    kn = k[n]
    offE = np.stack([np.broadcast_to(-(stag_E[q] * dx * kn) * scale, shape) for q in range(3)])
    offH = np.stack([np.broadcast_to(-(stag_H[q] * dx * kn) * scale, shape) for q in range(3)])
    P = int(np.prod(shape))
    f32 = lambda x: np.ascontiguousarray(np.broadcast_to(x, (3, *shape)).reshape(3, P), dtype=np.float32)  # noqa: E731
    return f32(E), f32(Hf), f32(offE), f32(offH)


def _interp_renormalised(arr: np.ndarray, pu: np.ndarray, pv: np.ndarray) -> np.ndarray:
    """Bilinear sampling of a 2-D array at fractional indices (fdtdx/core/misc.py:363-390): the
    floor / ceil neighbours, weights prod(1 - |index - point|), neighbours outside the array
    dropped, and the sum divided by (sum of the kept weights + 1e-8)."""
    acc = np.zeros_like(pu)
    wsum = np.zeros_like(pu)
    for iu in (np.floor(pu), np.ceil(pu)):
        for iv in (np.floor(pv), np.ceil(pv)):
            ok = (iu >= 0) & (iu < arr.shape[0]) & (iv >= 0) & (iv < arr.shape[1])
            wgt = np.where(ok, (1.0 - np.abs(iu - pu)) * (1.0 - np.abs(iv - pv)), 0.0)
            acc += wgt * arr[np.where(ok, iu, 0).astype(np.int64), np.where(ok, iv, 0).astype(np.int64)]
            wsum += wgt
    return acc / (wsum + 1e-8)


def _tilted_plane_profiles(src: LinearlyPolarizedPlaneSource, arrays: ArrayContainer, config: SimulationConfig):
    """Incident profiles and Yee time offsets of a plane source tilted by azimuth / elevation.

    Restates LinearlyPolarizedPlaneSource.apply (linear_polarization.py:168-330) on a uniform
    grid: the plane's cells, taken relative to its centre, are projected onto the plane normal
    to the tilted wave vector k, written in the in-plane basis u = (e_h - (e_h.k) k) / |...| and
    v = sign k x u, and the transverse profile is sampled there bilinearly.  The offsets are
    -(r . k) n / (c dt) with r the Yee position of each component relative to the plane's
    centre (calculate_time_offset_yee, fdtdx/core/grid.py:720-880), so they vary across the
    plane.  The kernels read per-cell profiles and offsets, so a tilted source needs no other
    device path than an untilted one.
    """
    n = src.propagation_axis
    h_ax, v_ax = src.horizontal_axis, src.vertical_axis
    shape = src.grid_shape
    dx, dt = config.uniform_spacing(), config.time_step_duration
    W, Hn = shape[h_ax], shape[v_ax]
    ch, cv = 0.5 * (W - 1), 0.5 * (Hn - 1)
    e_pol, h_pol, k = src.polarization_vectors()
    e_h = np.zeros(3)
    e_h[h_ax] = 1.0
    ub = e_h - (e_h @ k) * k
    ub = ub / np.linalg.norm(ub)
    vb = (1.0 if src.direction == "+" else -1.0) * np.cross(k, ub)
    w, hh = np.meshgrid(np.arange(W, dtype=np.float64), np.arange(Hn, dtype=np.float64), indexing="ij")
    pts = np.zeros((W, Hn, 3))
    pts[..., h_ax] = w - ch
    pts[..., v_ax] = hh - cv
    proj = pts - (pts @ k)[..., None] * k
    prof_hv = _interp_renormalised(src.amplitude_raw_hv(dx), proj @ ub + ch, proj @ vb + cv)
    prof = prof_hv.T if h_ax > v_ax else prof_hv
    amp = np.expand_dims(prof, axis=n)
    E = amp[None] * e_pol[:, None, None, None]
    Hf = amp[None] * h_pol[:, None, None, None]
    sl = (slice(None), *src.grid_slice)
    ie = arrays.inv_permittivities[sl].detach().double().cpu().numpy()
    if arrays.dispersive_c1 is not None:  # impedance, energy and offsets at the carrier (linear_polarization.py:186-211)
        ie = _carrier_inv_eps(ie, arrays, src.grid_slice, src, config)
    mu = arrays.inv_permeabilities
    im = mu[sl].detach().double().cpu().numpy() if isinstance(mu, torch.Tensor) else float(mu)
    E, Hf = _medium_scaling(src, ie, im, E, Hf, e_pol, h_pol)
    # Yee positions in the plane's frame: component q of E sits half a cell along axis q, of H
    # half a cell along the other two axes; the plane's centre is (ch, cv) cells across, 0 along n
    centre = np.zeros(3)
    centre[h_ax], centre[v_ax] = ch, cv
    idx = np.stack(np.meshgrid(*(np.arange(m, dtype=np.float64) for m in shape), indexing="ij"), axis=-1)
    ie0 = ie[0]
    im0 = im[0] if isinstance(im, np.ndarray) else im
    scale = (1.0 / np.sqrt(ie0 * im0)) / (constants.c * dt)

    def offsets(half_along):
        out = []
        for q in range(3):
            stag = np.array([0.5 if half_along(q, a) else 0.0 for a in range(3)])
            r = (idx + stag - centre) * dx
            out.append(-(r @ k) * scale)
        return np.stack(out)

    offE = offsets(lambda q, a: a == q)
    offH = offsets(lambda q, a: a != q)
    P = int(np.prod(shape))
    f32 = lambda x: np.ascontiguousarray(np.broadcast_to(x, (3, *shape)).reshape(3, P), dtype=np.float32)  # noqa: E731
    return f32(E), f32(Hf), f32(offE), f32(offH)


@dataclass
class DetectorTables:
    desc: N.DetectorDesc
    keep: list = field(default_factory=list)


def detector_tables(det, config: SimulationConfig) -> tuple[np.ndarray, np.ndarray | None]:
    """(slot, weights) for t in [-1, T]."""
    T = config.time_steps_total
    dt = config.time_step_duration
    on_list = det.on_list(config)
    ts = np.arange(-1, T + 1)
    if T == 0:
        return np.full(T + 2, -1, np.int32), None
    on = np.array([on_list[_jax_index(t, T)] for t in ts], bool)
    if isinstance(det, PhasorDetector):
        slot = np.where(on, 0, -1).astype(np.int32)
        on_arr = np.asarray(on_list, np.float64)
        if det.apodization is None:
            window = on_arr
        else:
            window = det.apodization.get_window(np.arange(T) * dt) * on_arr
        wsum = float(window.sum())
        if not math.isfinite(wsum) or wsum <= 0.0:
            raise Exception(f"Detector '{det.name}': the apodization window sums to {wsum} over the recorded "
                            "time steps; it must be finite and positive. Check that the window's support overlaps "
                            "the detector's active interval.")
        if det.scaling_mode == "continuous":
            scale = 2.0 / wsum
        elif det.scaling_mode == "pulse":
            scale = float(det.resolve_dft_stride(config))
        else:
            raise Exception(f"Invalid scaling mode: {det.scaling_mode=}")
        omegas = np.array([TWO_PI * wc.get_frequency() for wc in det.wave_characters])
        wt = np.array([window[_jax_index(t, T)] for t in ts])
        phase = omegas[None, :] * (ts[:, None] * dt)
        w = np.exp(1j * phase) * scale * wt[:, None]
        weights = np.empty((T + 2, len(omegas), 2), np.float32)
        weights[..., 0] = w.real
        weights[..., 1] = w.imag
        return slot, weights
    idx, counter = [-1] * T, 0
    for t in range(T):
        if on_list[t]:
            idx[t] = counter
            counter += 1
    slot = np.array([idx[_jax_index(t, T)] if on[q] else -1 for q, t in enumerate(ts)], np.int32)
    return slot, None


def build_detector(det, config: SimulationConfig) -> DetectorTables:
    d = N.DetectorDesc()
    st = det.grid_slice_tuple
    for a in range(3):
        d.lo[a], d.hi[a] = st[a]
    d.exact_interpolation = 1 if det.exact_interpolation else 0
    d.inverse = 1 if det.inverse else 0
    dx = config.uniform_spacing()
    if isinstance(det, PhasorDetector):
        d.kind = N.DET_PHASOR
        d.n_freq = len(det.wave_characters)
        if d.n_freq > N.MAX_FREQS:
            raise ValueError(f"at most {N.MAX_FREQS} frequencies per phasor detector")
        d.reduce_volume = 1 if det.reduce_volume else 0
        d.comp_mask = sum(1 << COMPONENTS.index(c) for c in det.recorded_components)
    elif isinstance(det, FieldDetector):
        d.kind = N.DET_FIELD
        d.reduce_volume = 1 if det.reduce_volume else 0
        d.comp_mask = sum(1 << COMPONENTS.index(c) for c in det.recorded_components)
    elif isinstance(det, PoyntingFluxDetector):
        d.kind = N.DET_FLUX
        d.reduce_volume = 1 if det.reduce_volume else 0
        d.keep_all = 1 if det.keep_all_components else 0
        d.flux_axis = det.propagation_axis if not det.keep_all_components else 0
        d.flux_sign = -1.0 if det.direction == "-" else 1.0
        d.cell_weight = dx * dx
        d.comp_mask = 63
    elif isinstance(det, EnergyDetector):
        d.kind = N.DET_ENERGY
        d.reduce_volume = 1 if det.reduce_volume else 0
        d.cell_weight = dx**3
        d.comp_mask = 63
    else:
        raise NotImplementedError(f"detector type {type(det).__name__} is not supported")
    slot, weights = detector_tables(det, config)
    keep = [slot]
    d.slot = slot.ctypes.data
    if weights is not None:
        keep.append(weights)
        d.weights = weights.ctypes.data
    return DetectorTables(d, keep)


class Scene:
    """The native description of one placed simulation and its plan."""

    def __init__(self, objects: ObjectContainer, arrays: ArrayContainer, config: SimulationConfig,
                 record_interfaces: bool = False):
        self.config = config
        self.desc = N.Desc()
        self._keep: list = []
        d = self.desc
        shape = objects.volume.grid_shape
        d.nx, d.ny, d.nz = shape
        d.n_steps_total = config.time_steps_total
        d.courant = config.courant_number
        d.n_eps = arrays.inv_permittivities.shape[0]
        mu = arrays.inv_permeabilities
        d.n_mu = mu.shape[0] if isinstance(mu, torch.Tensor) else 0
        d.inv_mu_scalar = 1.0 if isinstance(mu, torch.Tensor) else float(mu)
        if d.n_eps not in (1, 3, 9) or d.n_mu not in (0, 1, 3, 9):
            raise ValueError("material arrays have 1, 3 or 9 components")
        c1 = arrays.dispersive_c1
        if c1 is None and any(getattr(o.material, "is_dispersive", False) for o in objects.static_material_objects):
            raise ValueError("dispersive materials need the ADE coefficient arrays init_arrays allocates")
        d.n_poles = c1.shape[0] if c1 is not None else 0
        d.n_disp = c1.shape[1] if c1 is not None else 0
        self.dispersive = d.n_poles > 0
        d.n_sigma_E = arrays.electric_conductivity.shape[0] if arrays.electric_conductivity is not None else 0
        d.n_sigma_H = arrays.magnetic_conductivity.shape[0] if arrays.magnetic_conductivity is not None else 0
        # a 9-component material or conductivity runs that side's tensor half-steps
        self.full_tensor = 9 in (d.n_eps, d.n_mu, d.n_sigma_E, d.n_sigma_H)
        bloch: dict[int, list] = {}
        for b in objects.boundary_objects:
            side = 1 if b.direction == "+" else 0
            if isinstance(b, PeriodicBoundary):
                d.periodic[b.axis] = 1
                if b.needs_complex_fields:
                    bloch.setdefault(b.axis, []).append(b)
            elif isinstance(b, PerfectElectricConductor):
                d.pec_faces |= 1 << (2 * b.axis + side)
            elif isinstance(b, PerfectMagneticConductor):
                d.pmc_faces |= 1 << (2 * b.axis + side)
        # Bloch axes (bloch.py:59-94): the '+' ghost layer times exp(i k L), the '-' one times its
        # conjugate; the kernels carry the phase per axis, so both faces must carry the same one
        for ax, objs in bloch.items():
            phases = {o.direction: o.get_bloch_phase(shape, config.uniform_spacing()) for o in objs}
            if set(phases) != {"-", "+"} or abs(phases["-"] - phases["+"]) > 1e-12:
                raise NotImplementedError(f"axis {ax}: a Bloch phase must be set on both faces with the same vector")
            d.bloch_axes |= 1 << ax
            d.bloch_cos[ax] = phases["+"].real
            d.bloch_sin[ax] = phases["+"].imag
        self.complex_fields = d.bloch_axes != 0
        if self.dispersive and (self.complex_fields or 9 in (d.n_eps, d.n_sigma_E)):
            raise NotImplementedError("dispersive materials with complex (Bloch) fields or a full-tensor permittivity "
                                      "are not supported by the GB300 kernels")
        self._planar = None
        self._lam_ws = None
        self.pmls: list[PerfectlyMatchedLayer] = objects.pml_objects
        if len(self.pmls) > N.MAX_SLABS:
            raise ValueError("at most six PML slabs")
        d.n_slabs = len(self.pmls)
        for s, p in enumerate(self.pmls):
            lo, hi = p.grid_slice_tuple[p.axis]
            full = [(0, n) for n in shape]
            full[p.axis] = (lo, hi)
            if tuple(p.grid_slice_tuple) != tuple(full):
                raise NotImplementedError("a PML slab must span the whole domain transverse to its axis")
            if (p.direction == "-" and lo != 0) or (p.direction == "+" and hi != shape[p.axis]):
                raise NotImplementedError("a PML slab must touch its domain face")
            co = p.coefficients(config.uniform_spacing(), config.time_step_duration)
            tbl = np.ascontiguousarray(
                np.concatenate([co["a_E"], co["b_E"], co["inv_kappa_E"], co["a_H"], co["b_H"], co["inv_kappa_H"]]),
                dtype=np.float32,
            )
            self._keep.append(tbl)
            sd = d.slabs[s]
            sd.axis = p.axis
            sd.direction = -1 if p.direction == "-" else 1
            sd.thickness = p.thickness
            sd.kappa_is_one = 1 if p.kappa_is_one else 0
            sd.coef = tbl.ctypes.data
        self.sources = list(objects.sources)
        records = [tb for src in self.sources for tb in build_source(src, arrays, config)]
        if len(records) > N.MAX_SOURCES:
            raise ValueError(f"at most {N.MAX_SOURCES} source records (a tilted point dipole takes up to three)")
        d.n_sources = len(records)
        for s, tb in enumerate(records):
            self._keep.append(tb)
            d.sources[s] = tb.desc
        self.detectors = list(objects.forward_detectors)
        if len(self.detectors) > N.MAX_DETECTORS:
            raise ValueError(f"at most {N.MAX_DETECTORS} detectors")
        d.n_detectors = len(self.detectors)
        for q, det in enumerate(self.detectors):
            tb = build_detector(det, config)
            self._keep.append(tb)
            d.detectors[q] = tb.desc
        d.record_interfaces = 1 if record_interfaces else 0
        rec_dtype = torch.float32
        gc = config.gradient_config
        if gc is not None and gc.recorder is not None:
            rec_dtype = gc.recorder.storage_dtype
        d.recording_dtype = {torch.float32: 0, torch.bfloat16: 1, torch.float16: 2}[rec_dtype]
        tf = gc.recorder.time_filter if gc is not None and gc.recorder is not None else None
        d.rec_slots = 0
        if tf is not None and record_interfaces:
            T = config.time_steps_total
            store, ra, rb, rw = tf.tables(T)
            tabs = [np.asarray(store, dtype=np.int32), np.asarray(ra, dtype=np.int32),
                    np.asarray(rb, dtype=np.int32), np.asarray(rw, dtype=np.float32)]
            self._keep.extend(tabs)
            d.rec_slots = len(tf.save_steps(T))
            d.rec_store, d.rec_a, d.rec_b, d.rec_w = (x.ctypes.data for x in tabs)
        self._plan: int | None = None

    # ---- plan lifecycle
    @property
    def plan(self) -> int:
        if self._plan is None:
            lib = N.load()
            h = C.c_void_p()
            rc = lib.fdtd_plan_create(C.byref(self.desc), C.byref(h))
            N.check(rc, None, "fdtd_plan_create")
            self._plan = h.value
        return self._plan

    def close(self) -> None:
        if self._plan is not None:
            N.load().fdtd_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def footprint_bytes(self) -> int:
        return int(N.load().fdtd_footprint_bytes(C.byref(self.desc)))

    def launches_per_step(self) -> int:
        return int(N.load().fdtd_launches_per_step(self.plan))

    def interface_floats(self) -> int:
        return int(N.load().fdtd_interface_floats(self.plan))

    def tune(self, chunk: int = 0, vec: int = 0) -> None:
        """Launch shape of the register-queue update kernels (0 keeps the default)."""
        N.check(N.load().fdtd_plan_tune(self.plan, int(chunk), int(vec)), self.plan, "fdtd_plan_tune")

    def tune_shell(self, chunk: int = 0, vec: int = 0) -> None:
        """x planes per block and z cells per thread of the CPML shell kernels (0: default)."""
        N.check(N.load().fdtd_plan_tune_shell(self.plan, int(chunk), int(vec)), self.plan, "fdtd_plan_tune_shell")

    def tune_tma(self, enable: bool = True, tz: int = 0, ty: int = 0, stages: int = 0, chunk: int = 0) -> None:
        """Select the TMA-pipelined update kernels and their tile (0 keeps a default)."""
        N.check(N.load().fdtd_plan_tune_tma(self.plan, 1 if enable else 0, int(tz), int(ty), int(stages), int(chunk)),
                self.plan, "fdtd_plan_tune_tma")

    @property
    def uses_tma(self) -> bool:
        return bool(N.load().fdtd_plan_uses_tma(self.plan))

    def tune_shell_tma(self, mode: int = 2, tz: int = 0, chunk: int = 0) -> None:
        """Where the CPML slab cells run with a TMA core: 0 the register-queue shell kernel, 1 the
        x and y slabs in the TMA kernels (z boxes on the shell kernel), 2 the whole grid in one
        TMA launch (tile z extent ``tz``, 0: picked for nz), 3 split: the plain TMA kernels over
        the whole grid, then the slab cells' CPML corrections, one launch per axis, 4 the same
        with the z slabs' terms in the TMA tiles, 5 (the default where admitted) mode 4 for the E
        half-step and 3 for the H half-step (modes 3-5 split forward and reverse steps alike)."""
        N.check(N.load().fdtd_plan_tune_shell_tma(self.plan, int(mode), int(tz), int(chunk)), self.plan,
                "fdtd_plan_tune_shell_tma")

    @property
    def shell_tma(self) -> int:
        return int(N.load().fdtd_plan_shell_tma(self.plan))

    def status(self) -> None:
        """Raise if a kernel reported an error (a bounded pipeline wait that ran out)."""
        N.check(N.load().fdtd_plan_status(self.plan), self.plan, "fdtd_plan_status")

    # ---- buffers
    def _workspace(self, arrays: ArrayContainer) -> "PlanarFields":
        if self._planar is None or not self._planar.fits(arrays):
            self._planar = PlanarFields(arrays, self.pmls)
        return self._planar

    def buffers(self, arrays: ArrayContainer) -> N.Buffers:
        b = N.Buffers()
        f = arrays.fields
        if self.complex_fields:
            return self._complex_buffers(arrays)
        for t in (f.E, f.H, arrays.inv_permittivities):
            if not (t.is_cuda and t.is_contiguous() and t.dtype == torch.float32):
                raise ValueError("fields and materials must be contiguous float32 CUDA tensors")
        b.E, b.H = N.ptr(f.E), N.ptr(f.H)
        b.inv_eps = N.ptr(arrays.inv_permittivities)
        mu = arrays.inv_permeabilities
        b.inv_mu = N.ptr(mu) if isinstance(mu, torch.Tensor) else None
        b.sigma_E = N.ptr(arrays.electric_conductivity)
        b.sigma_H = N.ptr(arrays.magnetic_conductivity)
        for s, p in enumerate(self.pmls):
            b.psi_E[s][0], b.psi_E[s][1] = N.ptr(f.psi_E[p.name][0]), N.ptr(f.psi_E[p.name][1])
            b.psi_H[s][0], b.psi_H[s][1] = N.ptr(f.psi_H[p.name][0]), N.ptr(f.psi_H[p.name][1])
        for q, det in enumerate(self.detectors):
            st = arrays.detector_states[det.name]
            b.det_state[q] = N.ptr(next(iter(st.values())))
        if arrays.recording_state is not None:
            b.recording = N.ptr(arrays.recording_state.data["interfaces"])
        if self.dispersive:
            for t in (f.dispersive_P_curr, f.dispersive_P_prev, arrays.dispersive_c1, arrays.dispersive_c2,
                      arrays.dispersive_c3):
                if t is None or not (t.is_cuda and t.is_contiguous() and t.dtype == torch.float32):
                    raise ValueError("dispersive polarisation and coefficients must be contiguous float32 CUDA tensors")
            b.disp_P_curr, b.disp_P_prev = N.ptr(f.dispersive_P_curr), N.ptr(f.dispersive_P_prev)
            b.disp_c1, b.disp_c2, b.disp_c3 = (N.ptr(x) for x in (arrays.dispersive_c1, arrays.dispersive_c2,
                                                                   arrays.dispersive_c3))
        return b

    def _complex_buffers(self, arrays: ArrayContainer) -> N.Buffers:
        """Native buffers of a complex (Bloch) scene: the planar workspace's fields, psi and
        recording (real parts, then imaginary parts), the container's materials and states."""
        for t in (arrays.fields.E, arrays.fields.H, arrays.inv_permittivities):
            if not (t.is_cuda and t.is_contiguous()):
                raise ValueError("fields and materials must be contiguous CUDA tensors")
        ws = self._workspace(arrays)
        b = N.Buffers()
        b.E, b.H = N.ptr(ws.E), N.ptr(ws.H)
        b.inv_eps = N.ptr(arrays.inv_permittivities)
        mu = arrays.inv_permeabilities
        b.inv_mu = N.ptr(mu) if isinstance(mu, torch.Tensor) else None
        b.sigma_E = N.ptr(arrays.electric_conductivity)
        b.sigma_H = N.ptr(arrays.magnetic_conductivity)
        for s, p in enumerate(self.pmls):
            b.psi_E[s][0], b.psi_E[s][1] = N.ptr(ws.psi_E[p.name][0]), N.ptr(ws.psi_E[p.name][1])
            b.psi_H[s][0], b.psi_H[s][1] = N.ptr(ws.psi_H[p.name][0]), N.ptr(ws.psi_H[p.name][1])
        for q, det in enumerate(self.detectors):
            b.det_state[q] = N.ptr(next(iter(arrays.detector_states[det.name].values())))
        if ws.rec is not None:
            b.recording = N.ptr(ws.rec)
        return b

    def _run(self, arrays: ArrayContainer, call) -> None:
        """Runs a native call on the container's buffers (complex fields staged through the
        planar workspace and written back)."""
        if not self.complex_fields:
            call(self.buffers(arrays))
            return
        b = self.buffers(arrays)
        ws = self._workspace(arrays)
        ws.load(arrays)
        call(b)
        ws.store(arrays)

    def forward(self, arrays: ArrayContainer, t0: int, n_steps: int, graph: bool = True, stream=None,
                check_finite: bool = False) -> None:
        """Forward steps t0 .. t0+n_steps-1 in place.  ``check_finite`` scans E and H once after
        the last step; ``status()`` then raises ``NativeError`` (FDTD_ENONFINITE) when either
        holds a NaN or an infinity."""
        st = stream if stream is not None else torch.cuda.current_stream(arrays.device)
        flags = (N.FWD_GRAPH if graph else 0) | (N.FWD_CHECK_FINITE if check_finite else 0)

        def call(b):
            rc = N.load().fdtd_forward(self.plan, C.byref(b), int(t0), int(n_steps), flags, C.c_void_p(st.cuda_stream))
            N.check(rc, self.plan, "fdtd_forward")

        with torch.cuda.stream(st):
            self._run(arrays, call)

    def reverse(self, arrays: ArrayContainer, t_end: int, n_steps: int, stream=None) -> None:
        st = stream if stream is not None else torch.cuda.current_stream(arrays.device)

        def call(b):
            rc = N.load().fdtd_reverse(self.plan, C.byref(b), int(t_end), int(n_steps), C.c_void_p(st.cuda_stream))
            N.check(rc, self.plan, "fdtd_reverse")

        with torch.cuda.stream(st):
            self._run(arrays, call)

    def adjoint(self, arrays: ArrayContainer, lam: dict, t_end: int, n_steps: int, stream=None) -> None:
        """Backward loop of the reversible gradient on the native path (``fdtd_adjoint``).

        ``arrays`` holds the forward state at ``t_end`` and is reconstructed in place down to
        ``t_end - n_steps``.  ``lam`` holds the cotangents of that state: ``"E"``, ``"H"``,
        ``"psi_E"`` / ``"psi_H"`` (name -> (psi1, psi2)), ``"det"`` (detector name -> tensor
        of the state's layout, complex states with torch's convention), ``"grad_inv_eps"`` and
        ``"grad_inv_mu"`` (accumulated; either may be absent); all are updated in place.
        Complex (Bloch) fields and their cotangents (dL/dRe + i dL/dIm) are staged through
        planar workspaces.
        """
        st = stream if stream is not None else torch.cuda.current_stream(arrays.device)
        for key in ("E", "H"):
            t = lam[key]
            want = torch.complex64 if self.complex_fields else torch.float32
            if not (t.is_cuda and t.is_contiguous() and t.dtype == want):
                raise ValueError(f"cotangents must be contiguous {want} CUDA tensors")
        lw = None
        if self.complex_fields:
            if lam.get("grad_inv_mu") is not None:
                raise NotImplementedError("the inv_mu cotangent of complex (Bloch) fields is not supported")
            if self._lam_ws is None or not self._lam_ws.fits(lam):
                self._lam_ws = PlanarLam(lam, self.pmls)
            lw = self._lam_ws
        a = N.AdjointBuffers()
        src = lw if lw is not None else None
        a.lam_E, a.lam_H = (N.ptr(lw.E), N.ptr(lw.H)) if lw is not None else (N.ptr(lam["E"]), N.ptr(lam["H"]))
        for s, p in enumerate(self.pmls):
            pe = lw.psi_E[p.name] if lw is not None else lam["psi_E"][p.name]
            ph = lw.psi_H[p.name] if lw is not None else lam["psi_H"][p.name]
            a.lam_psi_E[s][0], a.lam_psi_E[s][1] = N.ptr(pe[0]), N.ptr(pe[1])
            a.lam_psi_H[s][0], a.lam_psi_H[s][1] = N.ptr(ph[0]), N.ptr(ph[1])
        del src
        dets = lam.get("det", {})
        for q, det in enumerate(self.detectors):
            t = dets.get(det.name)
            if t is not None and not (t.is_cuda and t.is_contiguous()):
                raise ValueError("detector cotangents must be contiguous CUDA tensors")
            a.lam_det[q] = N.ptr(t)
        a.grad_inv_eps = N.ptr(lam.get("grad_inv_eps"))
        a.grad_inv_mu = N.ptr(lam.get("grad_inv_mu"))

        def call(b):
            rc = N.load().fdtd_adjoint(self.plan, C.byref(b), C.byref(a), int(t_end), int(n_steps),
                                       C.c_void_p(st.cuda_stream))
            N.check(rc, self.plan, "fdtd_adjoint")

        with torch.cuda.stream(st):
            if lw is not None:
                lw.load(lam)
            self._run(arrays, call)
            if lw is not None:
                lw.store(lam)

    def adjoint_stored(self, arrays: ArrayContainer, states: list, t0: int, lam: dict, stream=None) -> None:
        """Backward loop over stored states (``fdtd_adjoint_stored``): ``states[q]`` is the
        ``FieldState`` of step ``t0 + q``; the transposed steps run from ``t0 + len(states) - 2``
        down to ``t0``.  ``arrays`` supplies the materials and detector states; ``lam`` as in
        ``adjoint`` (real fields; d/d inv_eps only)."""
        if self.complex_fields:
            raise NotImplementedError("the stored-state gradient of complex (Bloch) fields is not supported")
        if lam.get("grad_inv_mu") is not None:
            raise NotImplementedError("the stored-state gradient provides d/d inv_permittivities only")
        st = stream if stream is not None else torch.cuda.current_stream(arrays.device)
        n = len(states) - 1
        bufs = (N.Buffers * (n + 1))()
        for q, f in enumerate(states):
            bufs[q] = self.buffers(arrays.aset("fields", f))
        a = N.AdjointBuffers()
        for key in ("E", "H"):
            t = lam[key]
            if not (t.is_cuda and t.is_contiguous() and t.dtype == torch.float32):
                raise ValueError("cotangents must be contiguous float32 CUDA tensors")
        a.lam_E, a.lam_H = N.ptr(lam["E"]), N.ptr(lam["H"])
        for s, p in enumerate(self.pmls):
            a.lam_psi_E[s][0], a.lam_psi_E[s][1] = N.ptr(lam["psi_E"][p.name][0]), N.ptr(lam["psi_E"][p.name][1])
            a.lam_psi_H[s][0], a.lam_psi_H[s][1] = N.ptr(lam["psi_H"][p.name][0]), N.ptr(lam["psi_H"][p.name][1])
        dets = lam.get("det", {})
        for q, det in enumerate(self.detectors):
            a.lam_det[q] = N.ptr(dets.get(det.name))
        a.grad_inv_eps = N.ptr(lam.get("grad_inv_eps"))
        if self.dispersive:
            a.lam_P_curr, a.lam_P_prev = N.ptr(lam["P_curr"]), N.ptr(lam["P_prev"])
        rc = N.load().fdtd_adjoint_stored(self.plan, bufs, int(t0), int(n), C.byref(a), C.c_void_p(st.cuda_stream))
        N.check(rc, self.plan, "fdtd_adjoint_stored")


class PlanarFields:
    """The planar float32 workspace of a complex (Bloch) scene's state: E, H, the psi pairs and
    the interface recording as (2, ...) tensors, real parts first.  The native kernels work on
    one part at a time; ``load`` / ``store`` copy from / into the container's complex tensors."""

    def __init__(self, arrays: ArrayContainer, pmls):
        f = arrays.fields
        self.shapes = self._key(arrays)
        dev = f.E.device
        self.E = torch.empty((2, *f.E.shape), dtype=torch.float32, device=dev)
        self.H = torch.empty((2, *f.H.shape), dtype=torch.float32, device=dev)
        self.psi_E = {p.name: tuple(torch.empty((2, *t.shape), dtype=torch.float32, device=dev) for t in f.psi_E[p.name])
                      for p in pmls}
        self.psi_H = {p.name: tuple(torch.empty((2, *t.shape), dtype=torch.float32, device=dev) for t in f.psi_H[p.name])
                      for p in pmls}
        rec = arrays.recording_state
        self.rec = None
        if rec is not None:
            r = rec.data["interfaces"]
            self.rec = torch.empty((2, *r.shape), dtype=torch.float32, device=dev)

    @staticmethod
    def _key(arrays: ArrayContainer):
        f = arrays.fields
        rec = arrays.recording_state
        return (tuple(f.E.shape), tuple((k, tuple(a.shape)) for k, (a, _b) in f.psi_E.items()),
                None if rec is None else tuple(rec.data["interfaces"].shape))

    def fits(self, arrays: ArrayContainer) -> bool:
        return self._key(arrays) == self.shapes

    def _pairs(self, arrays: ArrayContainer):
        f = arrays.fields
        out = [(f.E, self.E), (f.H, self.H)]
        for k in self.psi_E:
            out += list(zip(f.psi_E[k], self.psi_E[k])) + list(zip(f.psi_H[k], self.psi_H[k]))
        if self.rec is not None:
            out.append((arrays.recording_state.data["interfaces"], self.rec))
        return out

    def load(self, arrays: ArrayContainer) -> None:
        for c, w in self._pairs(arrays):
            if not c.is_complex():
                raise ValueError("a scene with a Bloch phase needs complex fields (place it with place_objects)")
            r = torch.view_as_real(c)
            w[0].copy_(r[..., 0])
            w[1].copy_(r[..., 1])

    def store(self, arrays: ArrayContainer) -> None:
        for c, w in self._pairs(arrays):
            r = torch.view_as_real(c)
            r[..., 0].copy_(w[0])
            r[..., 1].copy_(w[1])


class PlanarLam:
    """The planar float32 workspace of a complex (Bloch) scene's cotangents: lam E, lam H and
    the psi cotangent pairs as (2, ...) tensors, dL/dRe parts first, then dL/dIm."""

    def __init__(self, lam: dict, pmls):
        self.key = self._key(lam)
        dev = lam["E"].device
        self.E = torch.empty((2, *lam["E"].shape), dtype=torch.float32, device=dev)
        self.H = torch.empty((2, *lam["H"].shape), dtype=torch.float32, device=dev)
        self.psi_E = {p.name: tuple(torch.empty((2, *t.shape), dtype=torch.float32, device=dev)
                                    for t in lam["psi_E"][p.name]) for p in pmls}
        self.psi_H = {p.name: tuple(torch.empty((2, *t.shape), dtype=torch.float32, device=dev)
                                    for t in lam["psi_H"][p.name]) for p in pmls}

    @staticmethod
    def _key(lam: dict):
        return (tuple(lam["E"].shape), tuple((k, tuple(a.shape)) for k, (a, _b) in lam["psi_E"].items()))

    def fits(self, lam: dict) -> bool:
        return self._key(lam) == self.key

    def _pairs(self, lam: dict):
        out = [(lam["E"], self.E), (lam["H"], self.H)]
        for k in self.psi_E:
            out += list(zip(lam["psi_E"][k], self.psi_E[k])) + list(zip(lam["psi_H"][k], self.psi_H[k]))
        return out

    def load(self, lam: dict) -> None:
        for c, w in self._pairs(lam):
            r = torch.view_as_real(c)
            w[0].copy_(r[..., 0])
            w[1].copy_(r[..., 1])

    def store(self, lam: dict) -> None:
        for c, w in self._pairs(lam):
            r = torch.view_as_real(c)
            r[..., 0].copy_(w[0])
            r[..., 1].copy_(w[1])
