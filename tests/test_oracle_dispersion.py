"""Dispersive (ADE) materials on the oracle (CPU): Lorentz and Drude poles.

The GB300 kernels run the ADE update in forward steps (tests/test_gpu_dispersion.py); the
oracle states the reference's ADE update (fdtd/update.py:316-350), its per-cell coefficients
(dispersion.py:789-857, fdtd/initialization.py:686-1000) and the source corrections at the
carrier frequency (dipole.py:150-193, linear_polarization.py:186-211, tfsf.py:21-141,
256-261), so that a kernel for them has its checker ready.  Pins:

* the Lorentz model of the reference's test is eps(omega) = 4.0 with a small positive
  imaginary part (tests/simulation/physics/test_dispersion.py:265-274), and the
  susceptibility recovered from the stored recurrence coefficients equals the continuous
  model's (the inversion is exact);
* the painted coefficients follow the materials' painting order, zeros where no pole is;
* one update of a uniform periodic box (zero curl) is E + inv_eps sum_p (P^n - P_hat) with
  P_hat = c1 P^n + c2 P^{n-1} + c3 E^n, and the polarisation shifts (P_hat, P^n);
* a semi-infinite Lorentz half-space transmits the Fresnel power of its eps(omega) within
  5% (test_dispersion.py:228-262; the oracle gives 2.1%); a Drude metal transmits nothing
  measurable (the reference's own check, |T - T_analytic| < 0.05) and absorbs the Fresnel
  fraction 1 - R within 10% (7.0% at 25 nm cells against a 16 nm power decay length);
* a plane source inside a uniform Lorentz medium injects the medium's impedance at the
  carrier: backward / forward flux < 2% (test_dispersion.py:329-360; the oracle gives 7e-7);
* per-axis Lorentz poles act on their own axis only: each polarisation matches the isotropic
  run with that axis' pole and its own Fresnel transmission
  (test_anisotropic_dispersion.py:203-244), and a Drude pole on x alone makes a hyperbolic
  medium that reflects x and passes y (test_anisotropic_dispersion.py:247-280);
* the broadband H-side filter leaks less of a Gaussian pulse's energy backwards than the
  carrier-only impedance (ratio below 0.85, test_dispersive_source.py:192-225);
* the library's own dispersive setup (painted coefficients, carrier-frequency source
  coefficients, the filtered E-side table of a plane source) equals the oracle's; the
  reversible gradient refuses a dispersive scene, and the oracle has no reversed step for one
  (fdtd/initialization.py:674-685).
"""

import ctypes
import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300.dispersion import compute_pole_coefficients_per_axis
from oracle import fdtd_oracle as O

C0 = 299792458.0
WL = 1e-6
ctypes_float = ctypes.c_float
OMEGA = 2 * math.pi * C0 / WL


def _lorentz():
    return fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=2 * OMEGA, damping=1e13, delta_epsilon=2.25),))


def _drude():
    return fx.DispersionModel(poles=(fx.DrudePole(plasma_frequency=5 * OMEGA, damping=0.05 * OMEGA),))


def _fresnel_t(eps: complex) -> float:
    n2 = np.sqrt(eps)
    return float(np.real(n2) * abs(2.0 / (1.0 + n2)) ** 2)


def test_lorentz_permittivity_and_discrete_susceptibility():
    eps = 1.0 + _lorentz().susceptibility(OMEGA)
    assert abs(eps.real - 4.0) < 0.05 and 0 < eps.imag < 0.01 * eps.real
    dt = 0.99 / math.sqrt(3) * 25e-9 / C0
    per_axis = fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=(2 * OMEGA, 1.5 * OMEGA, 3 * OMEGA),
                                                        damping=(1e13, 3e13, 0.0), delta_epsilon=(2.25, 1.0, 0.5)),
                                         fx.DrudePole(plasma_frequency=(5 * OMEGA, 0.0, 2 * OMEGA), damping=0.05 * OMEGA)))
    for model in (_lorentz(), _drude(), per_axis):
        c1, c2, c3, c4 = (torch.from_numpy(a) for a in compute_pole_coefficients_per_axis(model.poles, dt))
        assert torch.count_nonzero(c4) == 0  # no pole here has a numerator term
        for w in (0.6 * OMEGA, OMEGA, 1.7 * OMEGA):
            chi = O._chi_from_coefficients(c1, c2, c3, w, dt)  # (3,)
            want = model.susceptibility_axes(w)
            for ax in range(3):
                assert abs(complex(chi[ax]) - want[ax]) <= 1e-9 * max(abs(want[ax]), 1.0)


def _scene(mats, shape=(3, 3, 40), src=None, dets=(), steps=4, dtype=torch.float64, periodic_z=False):
    dx = 25e-9
    cfg = fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=shape)
    types = {"min_x": "periodic", "max_x": "periodic", "min_y": "periodic", "max_y": "periodic"}
    if periodic_z:
        types.update({"min_z": "periodic", "max_z": "periodic"})
    bc = fx.BoundaryConfig.from_uniform_bound(10, override_types=types)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values()) + list(mats)
    if src is not None:
        objs.append(src)
    objs += list(dets)
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg, O.OracleScene(objects, arrays, cfg, dtype)


def test_coefficients_follow_painting_order():
    lor = fx.Material(permittivity=1.0, dispersion=_lorentz())
    mats = [fx.UniformMaterialObject(name="lor", grid_slice_tuple=((0, 3), (0, 3), (5, 30)), material=lor),
            fx.UniformMaterialObject(name="glass", grid_slice_tuple=((0, 3), (0, 3), (20, 25)),
                                     material=fx.Material(permittivity=2.25), placement_order=1)]
    _, _, _, sc = _scene(mats)
    c1, c2, c3 = sc.disp
    assert c1.shape == (1, 1, 3, 3, 40)
    want = compute_pole_coefficients_per_axis(_lorentz().poles, sc.dt)
    for c, w in zip((c1, c2, c3), want):
        assert torch.allclose(c[0, 0, 1, 1, 10], torch.tensor(w[0, 0], dtype=torch.float64), rtol=1e-15)
        assert torch.count_nonzero(c[..., :5]) == 0 and torch.count_nonzero(c[..., 30:]) == 0
        assert torch.count_nonzero(c[..., 20:25]) == 0  # painted over by a material without poles
    # per-axis poles store three components
    aniso = fx.Material(dispersion=fx.DispersionModel(poles=(fx.DrudePole(plasma_frequency=(OMEGA, 0.0, 0.0),
                                                                          damping=1e13),)))
    _, _, _, sc3 = _scene([fx.UniformMaterialObject(name="a", grid_slice_tuple=((0, 3), (0, 3), (5, 30)),
                                                    material=aniso)])
    assert sc3.disp[0].shape == (1, 3, 3, 3, 40) and torch.count_nonzero(sc3.disp[2][0, 1]) == 0


def test_ade_update_formula():
    """Uniform fields in a periodic box have zero curl, so one E update is the ADE term alone."""
    mat = fx.Material(permittivity=2.0, dispersion=fx.DispersionModel(poles=_lorentz().poles + _drude().poles))
    _, _, _, sc = _scene([fx.UniformMaterialObject(name="m", grid_slice_tuple=((0, 3), (0, 3), (0, 8)), material=mat)],
                         shape=(3, 3, 8), periodic_z=True)
    st = sc.init_state()
    g = torch.Generator().manual_seed(4)
    E = torch.randn(3, 1, 1, 1, generator=g, dtype=torch.float64).expand(3, 3, 3, 8).clone()
    Pc = torch.randn(2, 3, 1, 1, 1, generator=g, dtype=torch.float64).expand(2, 3, 3, 3, 8).clone()
    Pp = torch.randn(2, 3, 1, 1, 1, generator=g, dtype=torch.float64).expand(2, 3, 3, 3, 8).clone()
    H = torch.zeros_like(E)
    E1, _, (Pn, Pc1) = O.update_E(sc, 0, E, H, st.psi_E, sc.inv_eps, P=(Pc, Pp))
    c1, c2, c3 = sc.disp
    P_hat = c1 * Pc + c2 * Pp + c3 * E
    assert torch.allclose(E1, E + sc.inv_eps * (Pc - P_hat).sum(0), rtol=1e-14, atol=1e-15)
    assert torch.equal(Pn, P_hat) and torch.equal(Pc1, Pc)


def _flux_run(mat, half=True, src_z=12, dets=(("t", 140),), e_pol=(1, 0, 0)):
    nz = 200
    cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(25e-9))
    vol = fx.SimulationVolume(shape=(3, 3, nz))
    bc = fx.BoundaryConfig.from_uniform_bound(10, override_types={"min_x": "periodic", "max_x": "periodic",
                                                                  "min_y": "periodic", "max_y": "periodic"})
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    if mat is not None:
        objs.append(fx.UniformMaterialObject(name="m", grid_slice_tuple=((0, 3), (0, 3), (100 if half else 0, nz)),
                                             material=mat))
    objs.append(fx.UniformPlaneSource(name="s", grid_slice_tuple=((0, 3), (0, 3), (src_z, src_z + 1)), direction="+",
                                      fixed_E_polarization_vector=e_pol, wave_character=fx.WaveCharacter(wavelength=WL)))
    for n, z in dets:
        objs.append(fx.PoyntingFluxDetector(name=n, grid_slice_tuple=((0, 3), (0, 3), (z, z + 1)), direction="+",
                                            reduce_volume=True))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    sc = O.OracleScene(objects, arrays, cfg, torch.float32)
    st = O.run(sc)
    spp = round(WL / (C0 * sc.dt))
    return {n: float(st.det[n]["poynting_flux"][:, 0].double()[-10 * spp:].mean()) for n, _ in dets}


def test_lorentz_and_drude_half_spaces():
    s0 = _flux_run(None, dets=(("t", 140), ("n", 60)))
    assert s0["t"] > 0 and s0["n"] > 0
    lor = _flux_run(fx.Material(permittivity=1.0, dispersion=_lorentz()))
    t_lor = _fresnel_t(1.0 + _lorentz().susceptibility(OMEGA))
    assert lor["t"] > 0 and abs(lor["t"] / s0["t"] - t_lor) / t_lor < 0.05, (lor["t"] / s0["t"], t_lor)
    dru = _flux_run(fx.Material(permittivity=1.0, dispersion=_drude()), dets=(("t", 140), ("n", 60)))
    t_dru = _fresnel_t(1.0 + _drude().susceptibility(OMEGA))
    assert t_dru < 0.05 and abs(dru["t"] / s0["t"] - t_dru) < 0.05
    absorbed = dru["n"] / s0["n"]  # net flux in front of the metal: 1 - R
    assert abs(absorbed - t_dru) / t_dru < 0.10, (absorbed, t_dru)


def test_embedded_source_matches_lorentz_impedance():
    r = _flux_run(fx.Material(permittivity=1.0, dispersion=_lorentz()), half=False, src_z=60,
                  dets=(("fwd", 90), ("bwd", 30)))
    assert r["fwd"] > 0 and abs(r["bwd"]) / r["fwd"] < 0.02


def test_library_dispersive_tables_match_oracle_and_reverse_is_refused():
    """The library's own restatement of the dispersive setup equals the oracle's: the painted
    ADE coefficients (a Lorentz slab painted over by glass), the carrier-frequency inverse
    permittivity of an electric dipole inside the slab, the plane source's impedance-divided
    H profile and its broadband-filtered E-side table.  The reversible gradient refuses the
    scene before any device work (fdtd.py:98-104), and the oracle has no reversed step."""
    from fdtdx_gb300.engine import Scene

    mat = fx.Material(permittivity=1.5, dispersion=_lorentz())
    pulse = fx.GaussianPulseProfile(spectral_width=fx.WaveCharacter(frequency=0.2 * C0 / WL),
                                    center_wave=fx.WaveCharacter(wavelength=WL))
    mats = [fx.UniformMaterialObject(name="m", grid_slice_tuple=((0, 3), (0, 3), (5, 30)), material=mat),
            fx.UniformMaterialObject(name="glass", grid_slice_tuple=((0, 3), (0, 3), (24, 27)),
                                     material=fx.Material(permittivity=2.25), placement_order=1)]
    src = fx.UniformPlaneSource(name="pl", grid_slice_tuple=((0, 3), (0, 3), (12, 13)), direction="+",
                                fixed_E_polarization_vector=(1, 0, 0), wave_character=fx.WaveCharacter(wavelength=WL),
                                temporal_profile=pulse)
    dip = fx.PointDipoleSource(name="d", grid_slice_tuple=((1, 2), (1, 2), (18, 19)), polarization=0,
                               wave_character=fx.WaveCharacter(wavelength=WL))
    # the float32 oracle: both store the coefficients in float32, as the reference does
    objects, arrays, cfg, sc = _scene(mats + [dip], src=src, steps=300, dtype=torch.float32)
    assert arrays.fields.dispersive_P_curr.shape == (1, 3, 3, 3, 40)
    for c, o in zip((arrays.dispersive_c1, arrays.dispersive_c2, arrays.dispersive_c3), sc.disp):
        assert torch.equal(c, o)
    scene = Scene(objects, arrays, cfg)
    assert scene.dispersive and scene.desc.n_poles == 1 and scene.desc.n_disp == 1
    recs = [scene.desc.sources[i] for i in range(scene.desc.n_sources)]
    plane = next(r for r in recs if r.kind == 1)
    dipole = next(r for r in recs if r.kind == 0)
    osrc = {s.obj.name: s for s in sc.sources}
    T = cfg.time_steps_total
    table = np.ctypeslib.as_array((ctypes_float * plane.n_e_table).from_address(plane.e_table))
    want = osrc["pl"].h_filter
    assert plane.n_e_table == T and np.max(np.abs(table - want)) <= 1e-6 * np.max(np.abs(want))
    inc_h = np.ctypeslib.as_array((ctypes_float * (3 * 9)).from_address(plane.inc_H)).reshape(3, 9)
    assert np.allclose(inc_h, osrc["pl"].H_inc.reshape(3, -1).numpy(), rtol=1e-6, atol=1e-9)
    local = float(osrc["d"].inv_local[0].reshape(-1)[0])
    assert math.isclose(dipole.coef, cfg.courant_number * local * dip.amplitude * dip.static_amplitude_factor,
                        rel_tol=1e-6)
    ie = arrays.inv_permittivities.clone().requires_grad_(True)
    with pytest.raises(NotImplementedError, match="dispersive"):
        fx.reversible_fdtd(arrays.aset("inv_permittivities", ie), objects, cfg)
    st = O.run(sc, 2)
    with pytest.raises(NotImplementedError):
        O.backward(sc, st)


def test_broadband_filter_reduces_backward_leakage():
    """A Gaussian pulse (15% bandwidth) from a plane source inside a strongly dispersive Lorentz
    medium: the H-side profile filtered by sqrt(eps(omega) / eps(omega_c)) leaks less
    pulse energy backwards (time-integrated |flux| behind / ahead) than the carrier-only
    impedance, by the reference's margin (ratio < 0.85;
    tests/simulation/physics/test_dispersive_source.py:192-225)."""
    nz = 200
    pulse = fx.GaussianPulseProfile(spectral_width=fx.WaveCharacter(frequency=0.15 * C0 / WL),
                                    center_wave=fx.WaveCharacter(wavelength=WL))
    model = fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=1.4 * OMEGA, damping=5e12,
                                                     delta_epsilon=1.5),))
    cfg = fx.SimulationConfig(time=180e-15, grid=fx.UniformGrid(25e-9))
    vol = fx.SimulationVolume(shape=(3, 3, nz))
    bc = fx.BoundaryConfig.from_uniform_bound(10, override_types={"min_x": "periodic", "max_x": "periodic",
                                                                  "min_y": "periodic", "max_y": "periodic"})
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="m", grid_slice_tuple=((0, 3), (0, 3), (0, nz)),
                                         material=fx.Material(permittivity=1.0, dispersion=model)))
    objs.append(fx.UniformPlaneSource(name="s", grid_slice_tuple=((0, 3), (0, 3), (60, 61)), direction="+",
                                      fixed_E_polarization_vector=(1, 0, 0), temporal_profile=pulse,
                                      wave_character=fx.WaveCharacter(wavelength=WL)))
    for name, z in (("fwd", 90), ("bwd", 30)):
        objs.append(fx.PoyntingFluxDetector(name=name, grid_slice_tuple=((0, 3), (0, 3), (z, z + 1)), direction="+",
                                            reduce_volume=True))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    leak = []
    for filtered in (True, False):
        sc = O.OracleScene(objects, arrays, cfg, torch.float32)
        assert sc.sources[0].h_filter is not None
        if not filtered:
            sc.sources[0].h_filter = None  # the carrier-only impedance path
        st = O.run(sc)
        fwd = float(st.det["fwd"]["poynting_flux"][:, 0].double().abs().sum())
        bwd = float(st.det["bwd"]["poynting_flux"][:, 0].double().abs().sum())
        assert fwd > 0 and bwd > 0
        leak.append(bwd / fwd)
    assert leak[0] / leak[1] < 0.85, leak


def test_per_axis_lorentz_half_space():
    """Per-axis Lorentz poles (delta_eps 2.25 on x, 0.75 on y and z): an x-polarised wave sees
    only chi_x and a y-polarised one only chi_y, so each run equals the isotropic run with that
    axis' pole (rel 1e-4) and transmits the Fresnel power of its own eps(omega) (5%), and the
    two transmissions differ (tests/simulation/physics/test_anisotropic_dispersion.py:203-244)."""
    w0 = 2.0 * OMEGA
    per_axis = fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=w0, damping=1e13,
                                                        delta_epsilon=(2.25, 0.75, 0.75)),))
    s0 = _flux_run(None)["t"]
    chi = per_axis.susceptibility_axes(OMEGA)
    t = {}
    for pol, de, e_pol in ((0, 2.25, (1, 0, 0)), (1, 0.75, (0, 1, 0))):
        iso = fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=w0, damping=1e13, delta_epsilon=de),))
        s_axis = _flux_run(fx.Material(permittivity=1.0, dispersion=per_axis), e_pol=e_pol)["t"]
        s_iso = _flux_run(fx.Material(permittivity=1.0, dispersion=iso), e_pol=e_pol)["t"]
        assert s_iso > 0 and abs(s_axis - s_iso) / s_iso < 1e-4
        t[pol] = s_axis / s0
        t_ref = _fresnel_t(1.0 + chi[pol])
        assert abs(t[pol] - t_ref) / t_ref < 0.05, (pol, t[pol], t_ref)
    assert abs(t[0] - t[1]) > 0.02


def test_hyperbolic_drude_medium_is_polarisation_selective():
    """A Drude pole on x only (omega_p = 5 omega, gamma = 0.05 omega): Re eps_x < 0 < eps_y, so
    the x polarisation reflects like a metal and the y polarisation passes, each at its Fresnel
    value within 0.05, and T_y - T_x > 0.8 (test_anisotropic_dispersion.py:247-280)."""
    model = fx.DispersionModel(poles=(fx.DrudePole(plasma_frequency=(5 * OMEGA, 0.0, 0.0), damping=0.05 * OMEGA),))
    chi = model.susceptibility_axes(OMEGA)
    assert (1.0 + chi[0]).real < 0 < (1.0 + chi[1]).real
    mat = fx.Material(permittivity=1.0, dispersion=model)
    s0 = _flux_run(None)["t"]
    t_x = _flux_run(mat, e_pol=(1, 0, 0))["t"] / s0
    t_y = _flux_run(mat, e_pol=(0, 1, 0))["t"] / s0
    assert abs(t_x - _fresnel_t(1.0 + chi[0])) < 0.05 and abs(t_y - _fresnel_t(1.0 + chi[1])) < 0.05
    assert t_y - t_x > 0.8


def test_pole_model_kats():
    """The pole models' closed forms and coefficient rules (tests/unit/test_dispersion.py:48-200)."""
    lor = fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=2e15, damping=1e13, delta_epsilon=3.5),))
    chi0 = lor.susceptibility(0.0)
    assert abs(chi0.imag) < 1e-18 and math.isclose(chi0.real, 3.5, rel_tol=1e-12)
    m = fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=1.5e15, damping=5e13, delta_epsilon=1.7),))
    for w in (0.3e15, 0.9e15, 1.4e15, 2.5e15):
        want = 1.7 * 1.5e15**2 / (1.5e15**2 - w**2 - 1j * 5e13 * w)
        assert abs(m.susceptibility(w) - want) <= 1e-12 * abs(want)
    d = fx.DispersionModel(poles=(fx.DrudePole(plasma_frequency=9e15, damping=1.5e13),))
    for w in (0.5e15, 2e15, 5e15):
        want = -(9e15**2) / (w**2 + 1j * 1.5e13 * w)
        assert abs(d.susceptibility(w) - want) <= 1e-12 * abs(want)
    p = fx.LorentzPole(resonance_frequency=2e15, damping=3e13, delta_epsilon=1.5)
    c1, c2, c3, c4 = compute_pole_coefficients_per_axis((p,), 5e-18)
    assert c4.shape == c1.shape and (c4 == 0).all()
    den = 1.0 + 0.5 * 3e13 * 5e-18
    assert np.allclose(c1[0], (2.0 - (2e15 * 5e-18) ** 2) / den, rtol=1e-12)
    assert np.allclose(c2[0], -(1.0 - 0.5 * 3e13 * 5e-18) / den, rtol=1e-12)
    assert np.allclose(c3[0], 1.5 * 2e15**2 * (5e-18) ** 2 / den, rtol=1e-12)
    q = fx.DrudePole(plasma_frequency=1e16, damping=1e14)
    c1, _, c3, _ = compute_pole_coefficients_per_axis((q,), 2e-18)
    den = 1.0 + 0.5 * 1e14 * 2e-18
    assert np.allclose(c1[0], 2.0 / den, rtol=1e-12) and np.allclose(c3[0], 1e32 * 4e-36 / den, rtol=1e-12)
    _, c2, _, _ = compute_pole_coefficients_per_axis((fx.LorentzPole(resonance_frequency=1e15, damping=1e13,
                                                                  delta_epsilon=2.0),), 1e-17)
    assert abs(c2[0, 0] + 1.0) < 2e-4
    slow = fx.LorentzPole(resonance_frequency=1e15, damping=1e10, delta_epsilon=2.0)
    with pytest.raises(ValueError, match=r"omega_0 \* dt"):
        compute_pole_coefficients_per_axis((slow,), 2.0 / 1e15)
    assert np.isfinite(compute_pole_coefficients_per_axis((slow,), 1.9 / 1e15)[0]).all()
    inert = fx.LorentzPole(resonance_frequency=3e17, damping=3e17, delta_epsilon=0.0)
    c1, c2, c3, _ = compute_pole_coefficients_per_axis((inert,), 1e-17)
    assert (c3 == 0).all() and np.isfinite(c1).all() and np.isfinite(c2).all()
    assert not fx.Material(permittivity=2.25).is_dispersive
    assert not fx.Material(dispersion=fx.DispersionModel()).is_dispersive
    assert fx.Material(dispersion=m).is_dispersive
