"""Analytic physics on the oracle (CPU, float32): the reference's simulation-tier checks
replayed on the restatement, so its physics is pinned beyond internal consistency.

* plane-wave wavenumber k = 2 pi n / lambda from the phasor phase between two planes, and
  the wave impedance |Ex| / |Hy| = 1 / n in fdtdx's normalised units (E is stored as
  E_SI / eta0), in vacuum and in eps_r = 4
  (tests/simulation/physics/test_plane_wave.py:185-241, 5%);
* Fresnel power transmission at normal incidence T = 4 n1 n2 / (n1 + n2)^2 from the
  time-averaged Poynting flux behind a vacuum / eps_r = 4 interface, normalised by a vacuum
  run (tests/simulation/physics/test_fresnel.py:150-244, 5%);
* a phasor flux plane equals the time-averaged time-domain flux over the same gated window
  (tests/simulation/physics/test_phasor_poynting_flux.py:90-138, 2%; the reference reports
  about 0.02%, the oracle gives 0.018%);
* the skin-depth attenuation in a sigma = 1e4 S/m conductor from the exact complex
  dispersion relation (tests/simulation/physics/test_skin_depth.py:60-276, 10%; the oracle
  gives 3.5%);
* total reflection from a PEC or PMC wall: zero net time-averaged flux of the standing wave
  against a PML-terminated run (tests/simulation/physics/boundaries/test_pec_reflection.py,
  test_pmc_reflection.py, 5%);
* a broadband pulse's stack transmission against single-frequency runs at three wavelengths
  (tests/simulation/fdtd/test_pulsed_vs_cw.py, 5%; the oracle gives 1.8-2.6%);
* a uniform plane source is linear in its amplitude factor and uniform across the periodic
  cross-section (tests/simulation/physics/sources/test_plane_source.py:108-146);
* birefringence in eps = diag(2.25, 4, 1): k and impedance 1/n of the ordinary (x) and
  extraordinary (y) polarisations (tests/simulation/physics/test_birefringence.py, 5%);
* point-dipole radiation: outward flux through six planes, x / y symmetry and a weaker axial
  flux for a z-dipole, the minimum along x for an x-dipole, a 45-degree tilted dipole's
  x = z, y > x pattern at equal total power, the magnetic dipole's dual pattern, and n times
  the vacuum power in a uniform dielectric
  (tests/simulation/physics/sources/test_dipole_radiation.py:138-312,
  test_dipole_magnetic.py:131-190, test_dipole_green_function.py:175-208, 40^3 box);
* the paraxial width of a Gaussian plane source's beam four cells downstream
  (tests/simulation/physics/sources/test_gaussian_source.py:148-219, 10%);
* mixed boundaries (PEC on x, PMC on y, both) with CPML along z keep free-space k and
  impedance (tests/simulation/physics/boundaries/test_mixed_boundaries.py, 5%);
* a TFSF plane injects one way: flux behind it below 1e-3 of the flux ahead;
* PEC walls put the standing wave's E node at the wall, PMC walls its antinode
  (tests/simulation/physics/boundaries/test_pec_pmc_symmetry.py:168-215).

The plane-wave checks use the reference's quasi-1D domains: 3 x 3 periodic cells across,
CPML along z, a +z uniform plane source with Ex polarisation (the default CW profile unless
stated).
"""

import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from oracle import fdtd_oracle as O

C0 = 299792458.0
WL = 1e-6
TOL = 0.05


def _domain(dx: float, nz: int, eps_fill: float | None = None, eps_half_from: int | None = None):
    cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(3, 3, nz))
    bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                           boundary_type_miny="periodic", boundary_type_maxy="periodic",
                           thickness_grid_minz=10, thickness_grid_maxz=10)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    if eps_fill is not None:
        objs.append(fx.UniformMaterialObject(name="fill", grid_slice_tuple=((0, 3), (0, 3), (0, nz)),
                                             material=fx.Material(permittivity=eps_fill)))
    if eps_half_from is not None:
        objs.append(fx.UniformMaterialObject(name="half", grid_slice_tuple=((0, 3), (0, 3), (eps_half_from, nz)),
                                             material=fx.Material(permittivity=4.0)))
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, 3), (0, 3), (12, 13)), direction="+",
                                      fixed_E_polarization_vector=(1, 0, 0),
                                      wave_character=fx.WaveCharacter(wavelength=WL)))
    return cfg, objs


def _run(cfg, objs):
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    sc = O.OracleScene(objects, arrays, cfg, torch.float32)
    return sc, O.run(sc, sc.T)


@pytest.mark.parametrize("eps_r,sep", [(1.0, 5), (4.0, 3)])
def test_plane_wave_wavenumber_and_impedance(eps_r, sep):
    dx = 50e-9
    cfg, objs = _domain(dx, 80, eps_fill=eps_r if eps_r != 1.0 else None)
    wc = fx.WaveCharacter(wavelength=WL)
    for name, z in (("d1", 17), ("d2", 17 + sep)):
        objs.append(fx.PhasorDetector(name=name, grid_slice_tuple=((1, 2), (1, 2), (z, z + 1)), wave_characters=(wc,),
                                      components=("Ex", "Hy"), reduce_volume=True))
    sc, st = _run(cfg, objs)
    p1 = st.det["d1"]["phasor"].reshape(-1)
    p2 = st.det["d2"]["phasor"].reshape(-1)
    ex1, hy1, ex2 = complex(p1[0]), complex(p1[1]), complex(p2[0])
    assert abs(ex1) > 0 and abs(ex2) > 0
    n = math.sqrt(eps_r)
    dphi = (np.angle(ex2) - np.angle(ex1)) % (2 * math.pi)  # exp(+i w t) weights: the phase grows along +z
    k = dphi / (sep * dx)
    k_ref = 2 * math.pi * n / WL
    assert abs(k - k_ref) / k_ref < TOL, (k, k_ref)
    z = abs(ex1) / abs(hy1)
    assert abs(z - 1 / n) / (1 / n) < TOL, (z, 1 / n)


def _mean_flux(st, steps_per_period: int) -> float:
    f = st.det["flux"]["poynting_flux"][:, 0].double().numpy()
    return float(f[-10 * steps_per_period:].mean())


def test_fresnel_normal_incidence_transmission():
    dx = 25e-9
    nz = 200
    out = []
    for half in (None, 100):
        cfg, objs = _domain(dx, nz, eps_half_from=half)
        objs.append(fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((0, 3), (0, 3), (140, 141)), direction="+",
                                            reduce_volume=True))
        sc, st = _run(cfg, objs)
        spp = round(WL / (C0 * sc.dt))
        out.append(_mean_flux(st, spp))
    s0, st_ = out
    assert s0 > 0 and st_ > 0
    n1, n2 = 1.0, 2.0
    t_ref = 4 * n1 * n2 / (n1 + n2) ** 2
    t = st_ / s0
    assert abs(t - t_ref) / t_ref < TOL, (t, t_ref)
    r = 1 - t
    r_ref = ((n1 - n2) / (n1 + n2)) ** 2
    assert abs(r - r_ref) / r_ref < TOL, (r, r_ref)


def test_phasor_flux_equals_time_averaged_flux():
    """A phasor flux plane's 1/2 Re(E x H*) equals the time average of a co-located time-domain
    flux plane over the same gated steady-state window (25 periods in, 10 periods on), in
    front of a lossy slab (tests/simulation/physics/test_phasor_poynting_flux.py:90-138, 2%;
    the reference observes about 0.02%)."""
    dx = 50e-9
    cfg, objs = _domain(dx, 80)
    objs.append(fx.UniformMaterialObject(name="slab", grid_slice_tuple=((0, 3), (0, 3), (22, 26)),
                                         material=fx.Material(permittivity=4.0, electric_conductivity=300.0)))
    period = WL / C0
    sw = fx.OnOffSwitch(start_after_periods=25, on_for_periods=10, period=period)
    wc = fx.WaveCharacter(wavelength=WL)
    objs.append(fx.PoyntingFluxDetector(name="td", grid_slice_tuple=((0, 3), (0, 3), (20, 21)), direction="+",
                                        reduce_volume=True, switch=sw))
    objs.append(fx.PhasorPoyntingFluxDetector(name="fd", grid_slice_tuple=((0, 3), (0, 3), (20, 21)), direction="+",
                                              wave_characters=(wc,), switch=sw))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    st = O.run(sc, sc.T)
    td = float(st.det["td"]["poynting_flux"][:, 0].mean())
    fd_obj = [d for d in objects.detectors if d.name == "fd"][0]
    fd = float(fd_obj.compute_poynting_flux({"phasor": st.det["fd"]["phasor"]}, dx)[0])
    assert abs(td) > 0
    assert abs(fd - td) / abs(td) < 0.02, (fd, td)


def test_skin_depth_in_a_conductor():
    """A plane wave entering a sigma = 1e4 S/m, eps_r = 1 conductor decays with the attenuation
    alpha = Im((w / c0) sqrt(eps_r - i sigma / (w eps0))): the Ex phasor amplitude ratio of two
    planes 1 um apart inside it (tests/simulation/physics/test_skin_depth.py:60-276, 10%)."""
    dx = 50e-9
    nz = 90
    cfg = fx.SimulationConfig(time=80e-15, grid=fx.UniformGrid(dx))
    cfg_objs = _domain(dx, nz)[1]
    cfg_objs.append(fx.UniformMaterialObject(name="cond", grid_slice_tuple=((0, 3), (0, 3), (30, 80)),
                                             material=fx.Material(permittivity=1.0, electric_conductivity=1e4)))
    wc = fx.WaveCharacter(wavelength=WL)
    for name, z in (("d1", 35), ("d2", 55)):
        cfg_objs.append(fx.PhasorDetector(name=name, grid_slice_tuple=((1, 2), (1, 2), (z, z + 1)),
                                          wave_characters=(wc,), components=("Ex",), reduce_volume=True))
    sc, st = _run(cfg, cfg_objs)
    p1 = complex(st.det["d1"]["phasor"].reshape(-1)[0])
    p2 = complex(st.det["d2"]["phasor"].reshape(-1)[0])
    assert abs(p1) > 0 and abs(p2) > 0
    omega = 2 * math.pi * C0 / WL
    k = omega / C0 * np.sqrt(1.0 - 1j * 1e4 / (omega * O.EPS0))
    alpha_ref = abs(k.imag)
    alpha = -math.log(abs(p2) / abs(p1)) / (20 * dx)
    assert abs(alpha - alpha_ref) / alpha_ref < 0.10, (alpha, alpha_ref)


@pytest.mark.parametrize("wall", ["pec", "pmc"])
def test_conductor_wall_total_reflection(wall):
    """A PEC (or PMC) wall at z-max reflects all the power: the time-averaged flux of the
    standing wave in front of it vanishes against a PML-terminated run, R = 1 within 5%
    (tests/simulation/physics/boundaries/test_pec_reflection.py:150-175, test_pmc_reflection.py)."""
    dx = 50e-9
    flux = []
    for zmax in ("pml", wall):
        cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
        vol = fx.SimulationVolume(shape=(3, 3, 80))
        bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                               boundary_type_miny="periodic", boundary_type_maxy="periodic",
                               boundary_type_maxz=zmax, thickness_grid_minz=10, thickness_grid_maxz=10)
        objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
        objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, 3), (0, 3), (12, 13)), direction="+",
                                          fixed_E_polarization_vector=(1, 0, 0),
                                          wave_character=fx.WaveCharacter(wavelength=WL)))
        objs.append(fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((0, 3), (0, 3), (40, 41)), direction="+",
                                            reduce_volume=True))
        sc, st = _run(cfg, objs)
        flux.append(_mean_flux(st, round(WL / (C0 * sc.dt))))
    s_ref, s_wall = flux
    assert s_ref > 0
    r = 1.0 - s_wall / s_ref
    assert abs(r - 1.0) < 0.05, r


def _stack_run(profile, wave, wavelengths, with_stack: bool):
    dx = 25e-9
    cfg = fx.SimulationConfig(time=200e-15, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(3, 3, 200))
    bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                           boundary_type_miny="periodic", boundary_type_maxy="periodic",
                           thickness_grid_minz=10, thickness_grid_maxz=10)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    if with_stack:
        for name, (z0, z1), eps in (("l1", (80, 100), 2.25), ("l2", (100, 115), 6.25), ("l3", (115, 135), 4.0)):
            objs.append(fx.UniformMaterialObject(name=name, grid_slice_tuple=((0, 3), (0, 3), (z0, z1)),
                                                 material=fx.Material(permittivity=eps)))
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, 3), (0, 3), (12, 13)), direction="+",
                                      fixed_E_polarization_vector=(1, 0, 0), wave_character=wave,
                                      temporal_profile=profile))
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((1, 2), (1, 2), (160, 161)),
                                  wave_characters=tuple(fx.WaveCharacter(wavelength=w) for w in wavelengths),
                                  components=("Ex",), reduce_volume=True))
    _, st = _run(cfg, objs)
    return st.det["ph"]["phasor"].reshape(-1).abs().double().numpy()


def test_pulsed_spectrum_matches_cw_transmission():
    """The transmission of a three-layer stack from one broadband pulse (normalised by a run
    without the stack) matches single-frequency runs at 0.85, 1.0 and 1.15 um
    (tests/simulation/fdtd/test_pulsed_vs_cw.py:1-248, 5%)."""
    wls = [0.85e-6, 1.0e-6, 1.15e-6]
    pulse = fx.GaussianPulseProfile(spectral_width=fx.WaveCharacter(wavelength=3e-6),
                                    center_wave=fx.WaveCharacter(wavelength=1e-6))
    w0 = fx.WaveCharacter(wavelength=1e-6)
    t_pulse = _stack_run(pulse, w0, wls, True) / _stack_run(pulse, w0, wls, False)
    for q, wl in enumerate(wls):
        w = fx.WaveCharacter(wavelength=wl)
        cw = fx.SingleFrequencyProfile()
        t_cw = _stack_run(cw, w, [wl], True)[0] / _stack_run(cw, w, [wl], False)[0]
        assert abs(t_pulse[q] - t_cw) / t_cw < 0.05, (wl, t_pulse[q], t_cw)


def test_uniform_plane_source_linearity_and_uniformity():
    """Doubling a uniform plane source's static amplitude factor doubles the transmitted phasor
    (5%), and across a 5 x 5 periodic cross-section the phasor's amplitude and phase are uniform
    (1% and 0.02 rad) (tests/simulation/physics/sources/test_plane_source.py:108-146)."""
    dx = 50e-9
    wc = fx.WaveCharacter(wavelength=WL)
    amps = []
    for factor in (1.0, 2.0):
        cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
        vol = fx.SimulationVolume(shape=(5, 5, 80))
        bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                               boundary_type_miny="periodic", boundary_type_maxy="periodic",
                               thickness_grid_minz=10, thickness_grid_maxz=10)
        objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
        objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, 5), (0, 5), (12, 13)), direction="+",
                                          fixed_E_polarization_vector=(1, 0, 0), wave_character=wc,
                                          static_amplitude_factor=factor))
        objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((0, 5), (0, 5), (22, 23)), wave_characters=(wc,),
                                      components=("Ex",)))
        _, st = _run(cfg, objs)
        amps.append(st.det["ph"]["phasor"].reshape(5, 5).to(torch.complex128))
    a1, a2 = amps
    ratio = float(a2.abs().mean() / a1.abs().mean())
    assert abs(ratio - 2.0) / 2.0 < 0.05, ratio
    mag = a1.abs()
    assert float((mag - mag.mean()).abs().max() / mag.mean()) < 0.01
    ph = torch.angle(a1 / a1[0, 0])
    assert float(ph.abs().max()) < 0.02


@pytest.mark.parametrize("pol", [0, 1])
def test_birefringence_wavenumber_and_impedance(pol):
    """A diagonally anisotropic fill eps = diag(2.25, 4, 1): an x-polarised wave travels with
    k_o = 2 pi 1.5 / lambda and |Ex| / |Hy| = 1 / 1.5, a y-polarised one with k_e = 2 pi 2 /
    lambda and |Ey| / |Hx| = 1 / 2 (tests/simulation/physics/test_birefringence.py:1-300, 5%)."""
    dx, nz, sep = 50e-9, 80, 3
    cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(3, 3, nz))
    bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                           boundary_type_miny="periodic", boundary_type_maxy="periodic",
                           thickness_grid_minz=10, thickness_grid_maxz=10)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="fill", grid_slice_tuple=((0, 3), (0, 3), (0, nz)),
                                         material=fx.Material(permittivity=(2.25, 4.0, 1.0))))
    e_pol = (1, 0, 0) if pol == 0 else (0, 1, 0)
    wc = fx.WaveCharacter(wavelength=WL)
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, 3), (0, 3), (12, 13)), direction="+",
                                      fixed_E_polarization_vector=e_pol, wave_character=wc))
    comps = ("Ex", "Hy") if pol == 0 else ("Ey", "Hx")
    for name, z in (("d1", 17), ("d2", 17 + sep)):
        objs.append(fx.PhasorDetector(name=name, grid_slice_tuple=((1, 2), (1, 2), (z, z + 1)), wave_characters=(wc,),
                                      components=comps, reduce_volume=True))
    _, st = _run(cfg, objs)
    p1 = st.det["d1"]["phasor"].reshape(-1)
    p2 = st.det["d2"]["phasor"].reshape(-1)
    e1, h1, e2 = complex(p1[0]), complex(p1[1]), complex(p2[0])
    assert abs(e1) > 0 and abs(e2) > 0
    n = 1.5 if pol == 0 else 2.0
    k = ((np.angle(e2) - np.angle(e1)) % (2 * math.pi)) / (sep * dx)
    k_ref = 2 * math.pi * n / WL
    assert abs(k - k_ref) / k_ref < TOL, (k, k_ref)
    z = abs(e1) / abs(h1)
    assert abs(z - 1 / n) / (1 / n) < TOL, (z, 1 / n)


def _dipole_fluxes(pol: int, azimuth: float = 0.0, source_type: str = "electric", eps: float = 1.0) -> dict:
    """Time-averaged flux through six full-width planes 8 cells from a CW point dipole at the
    centre of a 40^3 CPML box (50 nm cells)."""
    n, off = 40, 8
    cfg = fx.SimulationConfig(time=60e-15, grid=fx.UniformGrid(50e-9))
    vol = fx.SimulationVolume(shape=(n, n, n))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(8), vol).values())
    c = n // 2
    if eps != 1.0:
        objs.append(fx.UniformMaterialObject(name="fill", grid_slice_tuple=((0, n),) * 3,
                                             material=fx.Material(permittivity=eps)))
    objs.append(fx.PointDipoleSource(name="dip", grid_slice_tuple=((c, c + 1),) * 3, polarization=pol,
                                     azimuth_angle=azimuth, source_type=source_type,
                                     wave_character=fx.WaveCharacter(wavelength=WL)))
    for ax in range(3):
        for side in "+-":
            st = [(0, n)] * 3
            pos = c + off if side == "+" else c - off
            st[ax] = (pos, pos + 1)
            objs.append(fx.PoyntingFluxDetector(name=f"{'xyz'[ax]}{side}", grid_slice_tuple=tuple(st), direction=side,
                                                fixed_propagation_axis=ax, reduce_volume=True))
    sc, st = _run(cfg, objs)
    spp = round(WL / (C0 * sc.dt))
    return {k: float(v["poynting_flux"][:, 0].double()[-10 * spp:].mean()) for k, v in st.det.items()}


def test_dipole_radiation_pattern():
    """A z-dipole radiates outward through all six planes, equally through +-x and +-y and less
    along its axis; an x-dipole radiates least along x and the same total power; a z-dipole
    tilted 45 degrees in azimuth sends equal power through the x and z planes, more through y,
    and the same total (tests/simulation/physics/sources/test_dipole_radiation.py:138-312, 10%,
    on a 40^3 box instead of 60^3)."""
    fz = _dipole_fluxes(2)
    total = sum(fz.values())
    assert all(v > 0 for v in fz.values()) and total > 0
    assert abs(fz["x+"] - fz["x-"]) / fz["x+"] < 0.1 and abs(fz["x+"] - fz["y+"]) / fz["x+"] < 0.1
    assert fz["z+"] < fz["x+"]
    fx_ = _dipole_fluxes(0)
    per_axis = [fx_[f"{a}+"] + fx_[f"{a}-"] for a in "xyz"]
    assert int(np.argmin(per_axis)) == 0
    assert abs(sum(fx_.values()) - total) / total < 0.1
    ft = _dipole_fluxes(2, azimuth=45.0)
    sx, sy, sz = (abs(ft[f"{a}+"]) + abs(ft[f"{a}-"]) for a in "xyz")
    assert abs(sx - sz) / sx < 0.1 and sy > sx
    assert abs(sum(ft.values()) - total) / total < 0.1
    # a magnetic z-dipole: the same pattern (E <-> H duality) and power within a factor of 10
    # (tests/simulation/physics/sources/test_dipole_magnetic.py:131-190)
    fm = _dipole_fluxes(2, source_type="magnetic")
    assert all(v > 0 for v in fm.values())
    assert abs(fm["x+"] - fm["x-"]) / fm["x+"] < 0.1 and abs(fm["x+"] - fm["y+"]) / fm["x+"] < 0.1
    assert fm["z+"] < fm["x+"]
    ratio = max(total, sum(fm.values())) / min(total, sum(fm.values()))
    assert ratio < 10
    # in a uniform eps_r = 2.25 the same dipole radiates n = 1.5 times the vacuum power
    # (tests/simulation/physics/sources/test_dipole_green_function.py:175-208, 5%; the oracle
    # gives 1.507)
    fd = _dipole_fluxes(2, eps=2.25)
    assert abs(sum(fd.values()) / total - 1.5) / 1.5 < 0.05, sum(fd.values()) / total


def test_gaussian_plane_source_beam_width():
    """A Gaussian plane source of radius 1.5 um (sigma_0 = radius / 3 = 500 nm) in a 100 x 100
    CPML box: four cells downstream, the RMS width of |Ex|^2 across the beam is the paraxial
    sigma(z) / sqrt(2) with sigma(z)^2 = sigma_0^2 + (lambda z / (2 pi sigma_0))^2, within 10%
    (tests/simulation/physics/sources/test_gaussian_source.py:148-219; a 40-cell z extent and
    60 fs instead of 80 cells and 120 fs; the oracle gives 3.6%)."""
    dx, n = 50e-9, 100
    cfg = fx.SimulationConfig(time=60e-15, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(n, n, 40))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(10), vol).values())
    wc = fx.WaveCharacter(wavelength=WL)
    objs.append(fx.GaussianPlaneSource(name="g", grid_slice_tuple=((0, n), (0, n), (12, 13)), direction="+",
                                       fixed_E_polarization_vector=(1, 0, 0), radius=1.5e-6, wave_character=wc))
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((0, n), (0, n), (16, 17)), wave_characters=(wc,),
                                  components=("Ex",)))
    _, st = _run(cfg, objs)
    ex = st.det["ph"]["phasor"].reshape(n, n).abs().double().numpy()
    c = n // 2
    prof = ex[:, c]
    assert prof[c] > 0
    x = (np.arange(n) - c) * dx
    rms = math.sqrt(float((x**2 * prof**2).sum() / (prof**2).sum()))
    s0 = 1.5e-6 / 3
    sigma = math.sqrt(s0**2 + (WL * 4 * dx / (2 * math.pi * s0)) ** 2)
    assert abs(rms - sigma / math.sqrt(2)) / (sigma / math.sqrt(2)) < 0.10, (rms, sigma / math.sqrt(2))


@pytest.mark.parametrize("walls", ["pec_x", "pmc_y", "pec_x_pmc_y"])
def test_mixed_boundaries_keep_free_space_propagation(walls):
    """PEC walls on x, PMC walls on y, or both, with CPML along z: an x-polarised plane wave
    (Ex, Hy, neither constrained by those walls) keeps k = k0 between two planes 5 cells apart
    and, with PMC walls, the impedance |Ex| / |Hy| = 1 (tests/simulation/physics/boundaries/
    test_mixed_boundaries.py:194-268, 384-430, 5%)."""
    dx, nz, wide, narrow = 50e-9, 80, 40, 3
    nx = wide if "pec" in walls else narrow
    ny = wide if "pmc" in walls else narrow
    types = {"min_x": "pec" if "pec" in walls else "periodic", "max_x": "pec" if "pec" in walls else "periodic",
             "min_y": "pmc" if "pmc" in walls else "periodic", "max_y": "pmc" if "pmc" in walls else "periodic"}
    cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(nx, ny, nz))
    objs = [vol] + list(fx.boundary_objects_from_config(
        fx.BoundaryConfig.from_uniform_bound(10, override_types=types), vol).values())
    wc = fx.WaveCharacter(wavelength=WL)
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, nx), (0, ny), (12, 13)), direction="+",
                                      fixed_E_polarization_vector=(1, 0, 0), wave_character=wc))
    for name, z in (("d1", 17), ("d2", 22)):
        objs.append(fx.PhasorDetector(name=name, grid_slice_tuple=((0, nx), (0, ny), (z, z + 1)), wave_characters=(wc,),
                                      reduce_volume=True))
    _, st = _run(cfg, objs)
    p1 = st.det["d1"]["phasor"].reshape(-1)
    p2 = st.det["d2"]["phasor"].reshape(-1)
    ex1, hy1, ex2 = complex(p1[0]), complex(p1[4]), complex(p2[0])
    assert abs(ex1) > 0 and abs(ex2) > 0
    k = ((np.angle(ex2) - np.angle(ex1)) % (2 * math.pi)) / (5 * dx)
    k0 = 2 * math.pi / WL
    assert abs(k - k0) / k0 < TOL, (k, k0)
    if "pmc" in walls:
        assert abs(hy1) > 0 and abs(abs(ex1) / abs(hy1) - 1.0) < TOL


@pytest.mark.parametrize("direction,eps", [("+", 1.0), ("-", 1.0), ("+", 2.25)])
def test_tfsf_plane_injects_one_way(direction, eps):
    """A TFSF plane inside a uniform medium sends its wave one way only: the time-averaged flux
    behind it is below 1e-3 of the flux ahead, in vacuum and in eps_r = 2.25, for both
    directions (the property tests/simulation/physics/test_dispersion.py:329-360 checks in a
    dispersive medium, here in non-dispersive ones; the oracle gives 1.4e-9 to 2.3e-8)."""
    dx, nz = 25e-9, 200
    cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(3, 3, nz))
    bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                           boundary_type_miny="periodic", boundary_type_maxy="periodic",
                           thickness_grid_minz=10, thickness_grid_maxz=10)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    if eps != 1.0:
        objs.append(fx.UniformMaterialObject(name="fill", grid_slice_tuple=((0, 3), (0, 3), (0, nz)),
                                             material=fx.Material(permittivity=eps)))
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, 3), (0, 3), (100, 101)), direction=direction,
                                      fixed_E_polarization_vector=(1, 0, 0), wave_character=fx.WaveCharacter(wavelength=WL)))
    for name, z in (("lo", 50), ("hi", 150)):
        objs.append(fx.PoyntingFluxDetector(name=name, grid_slice_tuple=((0, 3), (0, 3), (z, z + 1)), direction="+",
                                            reduce_volume=True))
    sc, st = _run(cfg, objs)
    spp = round(WL / (C0 * sc.dt))
    lo, hi = _mean_flux_named(st, "lo", spp), _mean_flux_named(st, "hi", spp)
    ahead, behind = (hi, lo) if direction == "+" else (-lo, hi)
    assert ahead > 0 and abs(behind) < 1e-3 * ahead, (ahead, behind)


def _mean_flux_named(st, name: str, steps_per_period: int) -> float:
    f = st.det[name]["poynting_flux"][:, 0].double().numpy()
    return float(f[-10 * steps_per_period:].mean())


@pytest.mark.parametrize("wall", ["pec", "pmc"])
def test_conductor_wall_standing_wave_nodes(wall):
    """A plane wave reflected by a PEC wall has its E node at the wall and an antinode a quarter
    wavelength away (|Ex| one cell from the wall / |Ex| at lambda / 4 below 0.2); a PMC wall
    swaps them (ratio above 5) (tests/simulation/physics/boundaries/test_pec_pmc_symmetry.py:
    168-215, 12.5 nm cells, 100 fs instead of 150 fs)."""
    dx, nz = 12.5e-9, 400
    cfg = fx.SimulationConfig(time=100e-15, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(3, 3, nz))
    bc = fx.BoundaryConfig(boundary_type_minx="periodic", boundary_type_maxx="periodic",
                           boundary_type_miny="periodic", boundary_type_maxy="periodic",
                           thickness_grid_minz=10, boundary_type_maxz=wall)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    wc = fx.WaveCharacter(wavelength=WL)
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, 3), (0, 3), (12, 13)), direction="+",
                                      fixed_E_polarization_vector=(1, 0, 0), wave_character=wc))
    for name, z in (("near", nz - 2), ("far", nz - 21)):
        objs.append(fx.PhasorDetector(name=name, grid_slice_tuple=((0, 3), (0, 3), (z, z + 1)), wave_characters=(wc,),
                                      components=("Ex",), reduce_volume=True))
    _, st = _run(cfg, objs)
    near = float(st.det["near"]["phasor"].abs().max())
    far = float(st.det["far"]["phasor"].abs().max())
    if wall == "pec":
        assert far > 0 and near / far < 0.2, (near, far)
    else:
        assert near > 0 and (far == 0 or near / far > 5.0), (near, far)
