"""Tilted point dipoles and tilted TFSF plane sources (CPU).

* the tilt map (fdtdx/core/linalg.py:90-160) of the product and of the oracle agree, and the
  reference's orientation checks hold (tests/unit/objects/sources/test_dipole.py:244-350):
  zero angles are the identity, the result is a unit vector, 90 degrees of azimuth turn a
  z-dipole into x, 45 degrees split it equally;
* the oracle's tilted dipole injects into several components of its one cell and the inverse
  update undoes it, electric and magnetic (test_dipole.py:273-345);
* the library's per-component dipole records carry the oracle's injection coefficients;
* the library's tilted plane-source tables (incident E / H profiles and per-cell Yee time
  offsets) equal the oracle's restatement of LinearlyPolarizedPlaneSource.apply
  (linear_polarization.py:168-330), on every propagation axis and direction, Gaussian and
  uniform, isotropic and diagonal media; the tilted formula reduces to the untilted tables at
  zero angles, and a tilted uniform source keeps a constant profile;
* in vacuum the tables are energy-normalised with equal E and H norms, tilted or not, and
  the raw Gaussian profile sums to 1 around its central peak;
* physics: a 30-degree TE plane wave, in a periodic cell two wavelengths of the transverse
  period wide (k_x L = 2 pi, so plain wrap halos carry it exactly), crosses a vacuum /
  eps_r = 4 interface with the Fresnel power transmission T = 0.854 (5%), and its phasor phase
  advances across the cell at k0 sin(theta) (tests/simulation/physics/boundaries/
  test_bloch_oblique.py:1-205 uses a Bloch boundary for the same check; a commensurate
  periodic cell needs none).
"""

import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import _native as N
from fdtdx_gb300 import engine
from fdtdx_gb300.objects import tilt_vector
from oracle import fdtd_oracle as O

C0 = 299792458.0


def _both(vec, az_deg, el_deg, axes):
    a = tilt_vector(vec, math.radians(az_deg), math.radians(el_deg), axes)
    b = O.tilt_vector(torch.tensor(vec, dtype=torch.float64), float(np.deg2rad(az_deg)), float(np.deg2rad(el_deg)),
                      axes).numpy()
    return a, b


def test_tilt_map_kats_and_agreement():
    for p in range(3):
        axes = ((p + 1) % 3, (p + 2) % 3, p)
        base = np.zeros(3)
        base[p] = 1.0
        for az, el in ((0, 0), (30, 0), (0, 20), (35, 20), (60, 25), (-40, 10), (90, 0), (45, 0)):
            a, b = _both(base, az, el, axes)
            assert np.allclose(a, b, atol=1e-14)
            assert math.isclose(np.linalg.norm(a), 1.0, rel_tol=1e-12)
        assert np.allclose(_both(base, 0, 0, axes)[0], base)
    z = np.array([0.0, 0.0, 1.0])
    a90 = tilt_vector(z, math.radians(90.0), 0.0, (0, 1, 2))
    assert abs(a90[2]) < 1e-12 and abs(a90[0]) + abs(a90[1]) > 0.99
    a45 = tilt_vector(z, math.radians(45.0), 0.0, (0, 1, 2))
    assert math.isclose(abs(a45[0]), abs(a45[2]), rel_tol=1e-12) and abs(a45[1]) < 1e-12
    # a non-unit input keeps its norm (the map rescales to the input's norm)
    v = np.array([0.3, -1.2, 2.0])
    assert math.isclose(np.linalg.norm(tilt_vector(v, 0.4, -0.3, (2, 0, 1))), np.linalg.norm(v), rel_tol=1e-12)


def _dipole_scene(pol, az, el, source_type="electric", aniso=False):
    dx = 50e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=30 * dt, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(10, 9, 8))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(2), vol).values())
    objs.append(fx.UniformMaterialObject(name="m", grid_slice_tuple=((3, 7), (3, 7), (2, 6)),
                                         material=fx.Material(permittivity=(2.0, 3.0, 4.0) if aniso else 2.5,
                                                              permeability=(1.5, 1.2, 1.8) if aniso else 1.0)))
    objs.append(fx.PointDipoleSource(name="d", grid_slice_tuple=((4, 5), (4, 5), (4, 5)), polarization=pol,
                                     azimuth_angle=az, elevation_angle=el, source_type=source_type,
                                     amplitude=1.3, wave_character=fx.WaveCharacter(wavelength=1e-6)))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


@pytest.mark.parametrize("source_type", ["electric", "magnetic"])
def test_oracle_tilted_dipole_injection(source_type):
    objects, arrays, cfg = _dipole_scene(2, 45.0, 0.0, source_type)
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    s = sc.sources[0]
    F = torch.zeros((3, *sc.inv_eps.shape[1:]), dtype=torch.float64)
    upd = O._source_update_E if source_type == "electric" else O._source_update_H
    mat = sc.inv_eps if source_type == "electric" else sc.inv_mu
    t = 10.0
    G = upd(sc, s, F, mat, t, False)
    assert G[2, 4, 4, 4] != 0 and (G[0, 4, 4, 4] != 0 or G[1, 4, 4, 4] != 0)
    rest = G.clone()
    rest[:, 4, 4, 4] = 0
    assert torch.count_nonzero(rest) == 0
    assert torch.allclose(upd(sc, s, G, mat, t, True), F, atol=1e-15)
    # 90 degrees of azimuth: nothing left in z
    objects, arrays, cfg = _dipole_scene(2, 90.0, 0.0, source_type)
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    G = upd(sc, sc.sources[0], F, sc.inv_eps if source_type == "electric" else sc.inv_mu, t, False)
    assert abs(G[2, 4, 4, 4].item()) < 1e-12 * abs(G[:, 4, 4, 4]).max().item()


@pytest.mark.parametrize("pol,az,el,source_type,aniso", [
    (2, 0.0, 0.0, "electric", False), (2, 35.0, 20.0, "electric", True), (0, 60.0, 25.0, "electric", False),
    (1, -30.0, 15.0, "magnetic", True), (2, 90.0, 0.0, "electric", True)])
def test_dipole_records_carry_oracle_coefficients(pol, az, el, source_type, aniso):
    """Each record's coefficient c * amplitude * inv_material[axis] * orientation[axis] times the
    step's profile value is the oracle's injection into that component."""
    objects, arrays, cfg = _dipole_scene(pol, az, el, source_type, aniso)
    src = objects.sources[0]
    recs = engine.build_source(src, arrays, cfg)
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    s = sc.sources[0]
    F = torch.zeros((3, *sc.inv_eps.shape[1:]), dtype=torch.float64)
    t = 17.0
    if source_type == "electric":
        G = O._source_update_E(sc, s, F, sc.inv_eps, t, False)
    else:
        G = O._source_update_H(sc, s, F, sc.inv_mu, t, False)
    amp = O.profile_amplitude(src.temporal_profile, torch.tensor(t, dtype=torch.float64) * sc.dt,
                              src.wave_character.get_period(), src.wave_character.phase_shift).item()
    assert abs(amp) > 1e-3
    got = np.zeros(3)
    for r in recs:
        assert r.desc.kind == N.SRC_DIPOLE and r.desc.magnetic == (1 if source_type == "magnetic" else 0)
        got[r.desc.component] += -r.desc.coef * amp
    want = G[:, 4, 4, 4].numpy()
    assert len(recs) == (1 if az == 0.0 and el == 0.0 else int(np.count_nonzero(src.orientation)))
    assert np.allclose(got, want, rtol=2e-7, atol=1e-7 * np.abs(want).max())


def _plane_scene(n, direction, az, el, kind, eps3):
    dx = 25e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=20 * dt, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(30, 26, 22))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(4), vol).values())
    objs.append(fx.UniformMaterialObject(name="m", grid_slice_tuple=((8, 20), (6, 18), (5, 15)),
                                         material=fx.Material(permittivity=(2.0, 3.0, 2.5) if eps3 else 2.25)))
    st = [(5, 25), (5, 21), (5, 17)]
    st[n] = (11, 12)
    epol = [0, 0, 0]
    epol[(n + 1) % 3] = 1
    cls = fx.GaussianPlaneSource if kind == "gauss" else fx.UniformPlaneSource
    kw = {"radius": 0.2e-6} if kind == "gauss" else {"amplitude": 2.0}
    objs.append(cls(name="s", grid_slice_tuple=tuple(st), direction=direction, fixed_E_polarization_vector=tuple(epol),
                    azimuth_angle=az, elevation_angle=el, wave_character=fx.WaveCharacter(wavelength=1e-6), **kw))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


@pytest.mark.parametrize("n", [0, 1, 2])
@pytest.mark.parametrize("direction", ["+", "-"])
@pytest.mark.parametrize("kind,eps3,az,el", [("gauss", False, 30.0, 0.0), ("gauss", True, 35.0, -20.0),
                                             ("uniform", True, 0.0, 20.0), ("uniform", False, -25.0, 10.0)])
def test_tilted_plane_tables_match_oracle(n, direction, kind, eps3, az, el):
    objects, arrays, cfg = _plane_scene(n, direction, az, el, kind, eps3)
    src = objects.sources[0]
    tabs = engine.plane_source_profiles(src, arrays, cfg)
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    s = sc.sources[0]
    for got, want in zip(tabs, (s.E_inc, s.H_inc, s.off_E, s.off_H)):
        w = want.reshape(3, -1).numpy()
        assert np.abs(got - w).max() <= 2e-7 * max(np.abs(w).max(), 1e-30)
    # the offsets vary across the plane along the tilt, and the E / H tables are not plane-constant
    assert np.ptp(tabs[2][(n + 1) % 3]) > 1.0 or np.ptp(tabs[2][(n + 2) % 3]) > 1.0


@pytest.mark.parametrize("n", [0, 1, 2])
def test_tilted_formula_reduces_to_untilted_tables(n):
    objects, arrays, cfg = _plane_scene(n, "-", 0.0, 0.0, "gauss", True)
    src = objects.sources[0]
    flat = engine.plane_source_profiles(src, arrays, cfg)
    general = engine._tilted_plane_profiles(src, arrays, cfg)
    for a, b in zip(flat, general):
        assert np.allclose(a, b, rtol=1e-6, atol=1e-6 * max(np.abs(a).max(), 1e-30))


def test_tilted_uniform_source_keeps_constant_profile():
    """A constant transverse profile stays constant under the tilted projection (uniform-grid
    analogue of test_linear_polarization.py:357-380)."""
    objects, arrays, cfg = _plane_scene(2, "-", 20.0, 7.0, "uniform", False)
    src = objects.sources[0]
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    E = sc.sources[0].E_inc
    mag = torch.linalg.vector_norm(E, dim=0)
    inside = mag > 1e-12
    assert inside.float().mean() > 0.9 and torch.allclose(mag[inside], mag[inside].max(), rtol=1e-6)
    e_pol = src.polarization_vectors()[0]
    assert abs(e_pol[1]) > 1e-3 or abs(e_pol[2]) > 1e-3  # E tilted out of the x axis


def test_oblique_fresnel_te_and_transverse_phase():
    wl, dx, nx, nz, theta = 1e-6, 25e-9, 80, 160, 30.0
    out = []
    for diel in (False, True):
        cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
        vol = fx.SimulationVolume(shape=(nx, 3, nz))
        bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                               boundary_type_miny="periodic", boundary_type_maxy="periodic",
                               thickness_grid_minz=10, thickness_grid_maxz=10)
        objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
        if diel:
            objs.append(fx.UniformMaterialObject(name="d", grid_slice_tuple=((0, nx), (0, 3), (80, nz)),
                                                 material=fx.Material(permittivity=4.0)))
        objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, nx), (0, 3), (14, 15)), direction="+",
                                          fixed_E_polarization_vector=(0, 1, 0), azimuth_angle=theta,
                                          wave_character=fx.WaveCharacter(wavelength=wl)))
        objs.append(fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((0, nx), (0, 3), (120, 121)), direction="+",
                                            reduce_volume=True))
        if not diel:
            objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((0, nx), (1, 2), (60, 61)), components=("Ey",),
                                          wave_characters=(fx.WaveCharacter(wavelength=wl),), reduce_volume=False))
        objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
        sc = O.OracleScene(objects, arrays, cfg, torch.float32)
        st = O.run(sc, sc.T)
        spp = round(wl / (C0 * sc.dt))
        f = st.det["flux"]["poynting_flux"][:, 0].double().numpy()
        out.append(float(f[-10 * spp:].mean()))
        if not diel:
            ph = st.det["ph"]["phasor"].reshape(-1).numpy().astype(np.complex128)
            step = np.angle(ph[1:] / ph[:-1])
            k_x = 2 * math.pi * math.sin(math.radians(theta)) / wl
            assert abs(step.mean() - k_x * dx) / (k_x * dx) < 0.01, (step.mean(), k_x * dx)
    s0, s1 = out
    assert s0 > 0 and s1 > 0
    th = math.radians(theta)
    tt = math.asin(math.sin(th) / 2.0)
    t_ref = (2.0 * math.cos(tt)) / math.cos(th) * (2.0 * math.cos(th) / (math.cos(th) + 2.0 * math.cos(tt))) ** 2
    assert abs(s1 / s0 - t_ref) / t_ref < 0.05, (s1 / s0, t_ref)


@pytest.mark.parametrize("n", [0, 1, 2])
@pytest.mark.parametrize("az,el", [(0.0, 0.0), (30.0, -15.0)])
def test_plane_tables_in_vacuum_are_energy_normalised(n, az, el):
    """In vacuum the incident H table has the E table's norm (impedance 1) and, with
    ``normalize_by_energy``, sum 0.5 (|E|^2 + |H|^2) over the plane is 1; the raw Gaussian
    profile sums to 1 and peaks at the centre (tests/unit/objects/sources/
    test_linear_polarization.py:102-164, 215-238)."""
    dx = 25e-9
    cfg = fx.SimulationConfig(time=10 * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(24, 22, 20))
    st = [(2, 22), (3, 20), (2, 18)]
    st[n] = (9, 10)
    src = fx.GaussianPlaneSource(name="g", grid_slice_tuple=tuple(st), direction="+", radius=0.15e-6,
                                 fixed_E_polarization_vector=tuple(1 if a == (n + 1) % 3 else 0 for a in range(3)),
                                 azimuth_angle=az, elevation_angle=el, wave_character=fx.WaveCharacter(wavelength=1e-6))
    objects, arrays, _, cfg, _ = fx.place_objects([vol, src], cfg, device="cpu")
    src = objects.sources[0]
    raw = src.amplitude_raw_hv(dx)
    W, H = raw.shape
    assert math.isclose(float(raw.sum()), 1.0, rel_tol=1e-12) and raw[W // 2, H // 2] == raw.max() > raw[0, 0]
    E, Hh, _, _ = engine.plane_source_profiles(src, arrays, cfg)
    E, Hh = E.astype(np.float64), Hh.astype(np.float64)
    assert math.isclose(np.linalg.norm(E), np.linalg.norm(Hh), rel_tol=1e-6)
    assert math.isclose(float(0.5 * ((E**2).sum() + (Hh**2).sum())), 1.0, rel_tol=1e-6)
