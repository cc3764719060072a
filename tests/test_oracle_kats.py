"""Pins the oracle to the known answers and invariants of the reference's own tests.

The reference (fdtdx) stores no golden field values; its tests hold known-answer
tests and invariants.  Each test below replays one of them against the oracle
(the CPU restatement the GPU kernels are checked against), citing the test it
restates.
"""

import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from oracle import fdtd_oracle as O


# --------------------------------------------------------------------------- curls


def test_curl_E_linear_field():
    """E_x = y, E_y = -x gives curl_z = -2 (tests/unit/core/physics/test_curl.py:162-183)."""
    n = 6
    X, Y, _ = torch.meshgrid(torch.arange(n), torch.arange(n), torch.arange(n), indexing="ij")
    E = torch.stack([Y.double(), -X.double(), torch.zeros(n, n, n, dtype=torch.float64)])
    curl, psi = O.curl_E(O.pad_fields(E, (True, True, True)), {}, [], True)
    assert curl.shape == (3, 6, 6, 6)
    assert torch.allclose(curl[2][:-1, :-1], torch.full_like(curl[2][:-1, :-1], -2.0), atol=0.1)
    assert not psi


@pytest.mark.parametrize("which", ["E", "H"])
def test_curl_zero_field(which):
    """tests/unit/core/physics/test_curl.py:186-201 (and the curl_H twin)."""
    F = torch.zeros(3, 4, 4, 4)
    fn = O.curl_E if which == "E" else O.curl_H
    curl, psi = fn(O.pad_fields(F, (False, False, False)), {}, [], True)
    assert torch.all(curl == 0) and not psi


def _mock_pml(name, axis, sl, n):
    z = torch.zeros(1)
    return O.OPml(name, axis, "-", sl, 1.0, 1.0, z, z, z, z, z, z)


def test_curl_E_pml_scatter_signs(monkeypatch):
    """a=0: curl_y -= corr_1, curl_z += corr_2 (tests/unit/core/physics/test_curl.py:204-256)."""
    n = 5
    sl = (slice(None), slice(None), slice(1, 4))
    calls = {}

    def fake(pml, d1, d2, p1, p2, is_curl_E, simulate_boundaries):
        calls.update(is_curl_E=is_curl_E, simulate=simulate_boundaries, p1=p1, p2=p2)
        o = torch.ones(n, n, 3)
        return 0.1 * o, 0.2 * o, 0.3 * o, 0.4 * o

    monkeypatch.setattr(O, "step_cpml", fake)
    psi = {"pml_x": (torch.zeros(n, n, 3), torch.zeros(n, n, 3))}
    curl, new = O.curl_E(O.pad_fields(torch.zeros(3, n, n, n), (False,) * 3), psi, [_mock_pml("pml_x", 0, sl, n)], False)
    assert calls["is_curl_E"] is True and calls["simulate"] is False
    assert torch.allclose(new["pml_x"][0], torch.full((n, n, 3), 0.3))
    assert torch.allclose(new["pml_x"][1], torch.full((n, n, 3), 0.4))
    assert torch.allclose(curl[1][sl], torch.full((n, n, 3), -0.1))
    assert torch.allclose(curl[2][sl], torch.full((n, n, 3), 0.2))


def test_curl_H_pml_scatter_signs(monkeypatch):
    """a=1: curl_z -= corr_1, curl_x += corr_2 (tests/unit/core/physics/test_curl.py:381-431)."""
    n = 5
    sl = (slice(None), slice(None), slice(1, 4))

    def fake(pml, d1, d2, p1, p2, is_curl_E, simulate_boundaries):
        assert is_curl_E is False and simulate_boundaries is True
        o = torch.ones(n, n, 3)
        return 0.5 * o, 0.6 * o, 0.7 * o, 0.8 * o

    monkeypatch.setattr(O, "step_cpml", fake)
    psi = {"pml_y": (torch.zeros(n, n, 3), torch.zeros(n, n, 3))}
    curl, new = O.curl_H(O.pad_fields(torch.zeros(3, n, n, n), (False,) * 3), psi, [_mock_pml("pml_y", 1, sl, n)], True)
    assert torch.allclose(curl[2][sl], torch.full((n, n, 3), -0.5))
    assert torch.allclose(curl[0][sl], torch.full((n, n, 3), 0.6))
    assert torch.allclose(new["pml_y"][0], torch.full((n, n, 3), 0.7))


def test_interpolation_block_matches_full_domain():
    """Interpolating a haloed sub-block equals slicing the full-domain interpolation
    (tests/unit/core/physics/test_curl.py:139-154)."""
    g = torch.Generator().manual_seed(0)
    E = torch.randn(3, 8, 9, 10, generator=g, dtype=torch.float64)
    H = torch.randn(3, 8, 9, 10, generator=g, dtype=torch.float64)
    fE, fH = O.interpolate_fields(O.pad_fields(E, (False,) * 3), O.pad_fields(H, (False,) * 3))
    gst = ((2, 5), (3, 7), (1, 6))
    block = (slice(None), *(slice(s - 1, e + 1) for s, e in gst))
    region = (slice(None), *(slice(s, e) for s, e in gst))
    bE, bH = O.interpolate_fields(torch.nn.functional.pad(E[block], (1, 1, 1, 1, 1, 1)),
                                  torch.nn.functional.pad(H[block], (1, 1, 1, 1, 1, 1)))
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    assert torch.allclose(bE[inner], fE[region], atol=1e-12)
    assert torch.allclose(bH[inner], fH[region], atol=1e-12)


# --------------------------------------------------------------------------- scenes


def _box_scene(boundary="pml", shape=(12, 13, 14), pml=3, sigma=False, steps=4, dtype=torch.float32, record=False):
    cfg = fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * 50e-9 / 299792458.0, grid=fx.UniformGrid(50e-9),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()) if record else None)
    vol = fx.SimulationVolume(shape=shape)
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(pml, boundary), vol).values())
    mat = fx.Material(permittivity=4.0, electric_conductivity=2e4 if sigma else 0.0,
                      magnetic_conductivity=3e4 if sigma else 0.0)
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((4, 8), (5, 9), (4, 9)), material=mat))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return O.OracleScene(objects, arrays, cfg, dtype=dtype)


def _seed(sc, seed=42):
    g = torch.Generator().manual_seed(seed)
    st = sc.init_state()
    E = torch.randn(st.E.shape, generator=g, dtype=sc.dtype) * 1e-3
    H = torch.randn(st.H.shape, generator=g, dtype=sc.dtype) * 1e-3
    E = O._walls(sc, E, sc.pec)
    H = O._walls(sc, H, sc.pmc)
    st.E, st.H = E, H
    return st


@pytest.mark.parametrize("boundary", ["periodic", "pec", "pmc", "pml"])
def test_time_reversal_one_step(boundary):
    """One forward then one backward step restores E, H at atol 1e-5 in float32
    (tests/simulation/fdtd/test_time_reversal.py:251-308)."""
    sc = _box_scene(boundary, pml=3 if boundary == "pml" else 1, dtype=torch.float32, record=boundary == "pml")
    st = _seed(sc)
    E0, H0 = st.E.clone(), st.H.clone()
    fwd = O.forward(sc, st, record_detectors=False, record_boundaries=boundary == "pml")
    bwd = O.backward(sc, fwd)
    assert torch.allclose(bwd.E, E0, atol=1e-5) and torch.allclose(bwd.H, H0, atol=1e-5)


def test_time_reversal_lossy_multistep_fp64():
    """10 forward + 10 backward steps with conductivity restore the fields to rel < 1e-9 in float64
    (tests/simulation/fdtd/test_time_reversal.py:330-401, 403-471)."""
    sc = _box_scene("periodic", pml=1, sigma=True, dtype=torch.float64, steps=10)
    st = _seed(sc)
    E0, H0 = st.E.clone(), st.H.clone()
    for _ in range(10):
        st = O.forward(sc, st, record_detectors=False)
    for _ in range(10):
        st = O.backward(sc, st)
    assert float((st.E - E0).abs().max() / E0.abs().max()) < 1e-9
    assert float((st.H - H0).abs().max() / H0.abs().max()) < 1e-9


def test_update_formulas(monkeypatch):
    """E' = E + c curl inv_eps; lossy (1-q) E / (1+q) with q = c sigma eta0 inv_eps / 2; the reverse
    undoes the forward (tests/unit/fdtd/test_update.py:288-314, 424-435)."""
    sc = _box_scene("periodic", pml=1, dtype=torch.float64)
    n = sc.shape
    curl = torch.full((3, *n), 2.0, dtype=torch.float64)
    monkeypatch.setattr(O, "curl_H", lambda *a, **k: (curl, {}))
    E = torch.ones((3, *n), dtype=torch.float64)
    ie = torch.ones((1, *n), dtype=torch.float64)
    sc.sources, sc.sigma_E = [], None
    out, _ = O.update_E(sc, 0, E, E, {}, ie)
    assert torch.allclose(out, E + sc.courant * curl * ie)
    sc.sigma_E = torch.full((1, *n), 1e-4, dtype=torch.float64)
    monkeypatch.setattr(O, "curl_H", lambda *a, **k: (torch.zeros_like(curl), {}))
    out, _ = O.update_E(sc, 0, 2 * E, E, {}, ie)
    half = sc.courant * sc.sigma_E * O.ETA0 * ie / 2
    assert torch.allclose(out, (1 - half) * 2 * E / (1 + half), rtol=1e-12)
    monkeypatch.setattr(O, "curl_H", lambda *a, **k: (curl, {}))
    fwd, _ = O.update_E(sc, 0, E, E, {}, ie)
    rev = O.update_E_reverse(sc, 0, fwd, E, {}, ie)
    assert torch.allclose(rev, E, atol=1e-12)


# --------------------------------------------------------------------------- PML


def test_pml_defaults_and_profiles():
    """Defaults and profile monotonicity (tests/unit/objects/boundaries/test_perfectly_matched_layer.py:62-300)."""
    p = fx.PerfectlyMatchedLayer(axis=0, direction="-")
    assert p.alpha_start > 0 and p.alpha_end == 0.0 and p.alpha_order == 1.0
    assert p.kappa_start == 1.0 and p.kappa_end == 1.0 and p.kappa_order == 3.0
    assert p.sigma_start == 0.0 and p.sigma_order == 3.0 and p.sigma_end is None
    p.place_on_grid(((0, 10), (0, 20), (0, 20)))
    co = O.pml_coefficients(p, 50e-9, 1e-16, torch.float32)
    expected = -(3.0 + 1) * math.log(1e-6) / (2 * O.ETA0 * 10 * 50e-9)
    assert math.isclose(co["sigma_end"], expected)
    assert co["a_E"].shape == (10, 1, 1)
    # "-" side: deepest cell first; the interface cell has zero conductivity (a = 0)
    a = co["a_E"].flatten()
    assert float(a[-1]) == 0.0 and float(co["a_H"].flatten()[-1]) == 0.0
    assert torch.all(a[:-1].abs() >= a[1:].abs())
    q = fx.PerfectlyMatchedLayer(axis=2, direction="+")
    q.place_on_grid(((0, 20), (0, 20), (14, 20)))
    cq = O.pml_coefficients(q, 50e-9, 1e-16, torch.float32)
    aq = cq["a_E"].flatten()
    assert cq["a_E"].shape == (1, 1, 6) and float(aq[0]) == 0.0 and float(cq["a_H"].flatten()[0]) == 0.0
    assert torch.all(aq[1:].abs() >= aq[:-1].abs())


# --------------------------------------------------------------------------- phasor


def test_phasor_semantics():
    """Accumulation, phase rotation and the 2/N continuous scale (tests/unit/objects/detectors/test_phasor.py:96-314)."""
    sc = _box_scene("periodic", pml=1, dtype=torch.float64, steps=8)
    d = fx.PhasorDetector(name="ph", grid_slice_tuple=((2, 4), (2, 4), (2, 4)),
                          wave_characters=(fx.WaveCharacter(wavelength=1.55e-6),), components=("Ex",))
    sc.detectors = [sc._setup_detector(d)]
    st = sc.init_state()
    E = torch.ones((3, *sc.shape), dtype=torch.float64)
    H = torch.zeros_like(E)
    one = O.update_detectors(sc, 0, E, H, H, st.det, sc.inv_eps, sc.inv_mu)
    two = O.update_detectors(sc, 1, E, H, H, one, sc.inv_eps, sc.inv_mu)
    same = O.update_detectors(sc, 0, E, H, H, one, sc.inv_eps, sc.inv_mu)
    p1, p2, p0 = one["ph"]["phasor"], two["ph"]["phasor"], same["ph"]["phasor"]
    assert torch.allclose(p1, torch.full_like(p1, 2.0 / sc.T))  # exp(0) * 2/N
    assert not torch.allclose(p1, p2)
    assert torch.allclose(p0.abs(), 2 * p1.abs())
    w = 2 * math.pi * 299792458.0 / 1.55e-6 * sc.dt
    assert torch.allclose(p2, p1 * (1 + complex(math.cos(w), math.sin(w))))


def test_flux_and_energy_reduce_to_physical_integrals():
    """Uniform Ex = 1, Hy = 1 in a periodic box: a reduced flux plane of 2 x 2 cells is the
    surface integral 4 dx^2 ('-' flips it; all components give (0, 0, 4 dx^2)); Ex = 1 alone
    gives 0.5 |E|^2 = 0.5 per cell and the volume integral 4 x 0.5 dx^3 over the 4 cells, and
    eps_r = 2 doubles it (tests/unit/objects/detectors/test_poynting_flux.py:306-326,
    test_energy.py:243-262)."""
    dx = 2e-7
    cfg = fx.SimulationConfig(time=3 * 0.99 / math.sqrt(3) * dx / 299792458.0, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(4, 4, 4))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(1, "periodic"),
                                                        vol).values())
    plane = ((1, 3), (1, 3), (2, 3))
    objs += [fx.PoyntingFluxDetector(name="fp", grid_slice_tuple=plane, direction="+"),
             fx.PoyntingFluxDetector(name="fm", grid_slice_tuple=plane, direction="-"),
             fx.PoyntingFluxDetector(name="fa", grid_slice_tuple=plane, direction="+", keep_all_components=True),
             fx.EnergyDetector(name="en", grid_slice_tuple=plane, reduce_volume=True),
             fx.EnergyDetector(name="ec", grid_slice_tuple=plane)]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    st = sc.init_state()
    E = torch.zeros(3, 4, 4, 4, dtype=torch.float64)
    H = torch.zeros_like(E)
    E[0], H[1] = 1.0, 1.0
    det = O.update_detectors(sc, 0, E, H, H, st.det, sc.inv_eps, sc.inv_mu)
    assert math.isclose(float(det["fp"]["poynting_flux"][0, 0]), 4 * dx**2, rel_tol=1e-12)
    assert math.isclose(float(det["fm"]["poynting_flux"][0, 0]), -4 * dx**2, rel_tol=1e-12)
    assert torch.allclose(det["fa"]["poynting_flux"][0], torch.tensor([0.0, 0.0, 4 * dx**2], dtype=torch.float64))
    Eonly = O.update_detectors(sc, 0, E, torch.zeros_like(E), torch.zeros_like(E), st.det, sc.inv_eps, sc.inv_mu)
    assert math.isclose(float(Eonly["en"]["energy"][0, 0]), 4 * 0.5 * dx**3, rel_tol=1e-12)
    assert torch.allclose(Eonly["ec"]["energy"][0], torch.full((2, 2, 1), 0.5, dtype=torch.float64))
    sc2 = O.OracleScene(objects, arrays.aset("inv_permittivities", torch.full((1, 4, 4, 4), 0.5)), cfg,
                        torch.float64)
    E2 = O.update_detectors(sc2, 0, E, torch.zeros_like(E), torch.zeros_like(E), sc2.init_state().det, sc2.inv_eps,
                            sc2.inv_mu)
    assert math.isclose(float(E2["en"]["energy"][0, 0]), 4 * 1.0 * dx**3, rel_tol=1e-12)
