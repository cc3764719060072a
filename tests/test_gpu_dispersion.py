"""Dispersive (ADE) materials on the GPU against the oracle.

Before each E half-step ``k_ade`` advances every pole's polarisation, P_hat = c1 P^n + c2
P^(n-1) + c3 E^n, and folds inv_eps sum_poles (P^n - P_hat) into E ahead of the E kernel
(fdtdx/fdtd/update.py:316-350).  Sources see the medium at their carrier, and a plane source's
E side injects the broadband impedance-corrected profile (fdtdx/objects/sources/tfsf.py:21-141).
Tolerance: relative L2 <= 1e-4 against the float32 oracle (float64 reported); the physics
checks follow the reference's tests/simulation/physics/test_dispersion.py.
"""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import _native as N
from fdtdx_gb300.engine import Scene
from oracle import fdtd_oracle as O
from tests.helpers import compare_states, log_result

pytestmark = pytest.mark.gpu
TOL = 1e-4
C0 = 299792458.0
WL = 1e-6
OMEGA = 2 * math.pi * C0 / WL


def _lorentz():
    return fx.DispersionModel(poles=(fx.LorentzPole(resonance_frequency=2 * OMEGA, damping=1e13, delta_epsilon=2.25),))


def _drude():
    return fx.DispersionModel(poles=(fx.DrudePole(plasma_frequency=5 * OMEGA, damping=0.05 * OMEGA),))


def _fresnel_t(eps: complex) -> float:
    n2 = np.sqrt(eps)
    return float(np.real(n2) * abs(2.0 / (1.0 + n2)) ** 2)


@pytest.mark.parametrize("per_axis", [False, True])
def test_dispersive_scene_matches_oracle(per_axis):
    """A Lorentz + Drude slab (two poles; per-axis parameters: three coefficient components)
    with electric conductivity, a Lorentz block painted over part of it, a pulsed plane source
    inside the slab (filtered E-side table), an electric dipole inside it (carrier-frequency
    amplitude), CPML on z (kappa != 1) and periodic x, y; flux, energy, phasor and field
    detectors.  run_fdtd (CUDA graph) against the oracle."""
    if per_axis:
        poles = (fx.LorentzPole(resonance_frequency=(2 * OMEGA, 1.5 * OMEGA, 3 * OMEGA), damping=(1e13, 3e13, 0.0),
                                delta_epsilon=(2.25, 1.0, 0.5)),
                 fx.DrudePole(plasma_frequency=(2 * OMEGA, 0.0, OMEGA), damping=0.05 * OMEGA))
    else:
        poles = _lorentz().poles + (fx.DrudePole(plasma_frequency=1.5 * OMEGA, damping=0.05 * OMEGA),)
    slab = fx.Material(permittivity=1.5, electric_conductivity=2e3, dispersion=fx.DispersionModel(poles=poles))
    dx = 25e-9
    nx, ny, nz = 12, 10, 90
    wc = fx.WaveCharacter(wavelength=WL)
    pulse = fx.GaussianPulseProfile(spectral_width=fx.WaveCharacter(frequency=0.2 * C0 / WL), center_wave=wc)
    cfg = fx.SimulationConfig(time=400 * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx))
    vol = fx.SimulationVolume(shape=(nx, ny, nz))
    bc = fx.BoundaryConfig.from_uniform_bound(8, override_types={"min_x": "periodic", "max_x": "periodic",
                                                                 "min_y": "periodic", "max_y": "periodic"},
                                              kappa_end=1.5)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs += [
        fx.UniformMaterialObject(name="slab", grid_slice_tuple=((0, nx), (0, ny), (20, 70)), material=slab),
        fx.UniformMaterialObject(name="blk", grid_slice_tuple=((3, 9), (2, 8), (40, 50)), placement_order=1,
                                 material=fx.Material(permittivity=2.0, dispersion=_lorentz())),
        fx.UniformPlaneSource(name="pl", grid_slice_tuple=((0, nx), (0, ny), (30, 31)), direction="+",
                              fixed_E_polarization_vector=(1, 1, 0), wave_character=wc, temporal_profile=pulse),
        fx.PointDipoleSource(name="d", grid_slice_tuple=((6, 7), (5, 6), (45, 46)), polarization=2, wave_character=wc,
                             temporal_profile=pulse),
        fx.PoyntingFluxDetector(name="fl", grid_slice_tuple=((0, nx), (0, ny), (60, 61)), direction="+"),
        fx.EnergyDetector(name="en", grid_slice_tuple=((0, nx), (0, ny), (35, 55)), reduce_volume=True),
        fx.PhasorDetector(name="ph", grid_slice_tuple=((0, nx), (0, ny), (38, 52)), wave_characters=(wc,)),
        fx.FieldDetector(name="f", grid_slice_tuple=((0, nx), (0, ny), (65, 66)), components=("Ex", "Hy")),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cuda")
    assert arrays.dispersive_c1.shape == (2, 3 if per_axis else 1, nx, ny, nz)
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    res = [O.run(O.OracleScene(objects, arrays, cfg, dt)) for dt in (torch.float32, torch.float64)]
    assert res[1].det["en"]["energy"].abs().max() > 0
    compare_states(f"dispersion_{'per_axis' if per_axis else 'isotropic'}", out, res[0], res[1], TOL)


def _gpu_flux(mat, half=True, src_z=12, dets=(("t", 140),)):
    """The oracle test's half-space run on the GPU: periodic 3 x 3 x 200 column, CW plane wave
    at 1 um from z = src_z, the material from z = 100 (or everywhere), time-averaged flux."""
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
                                      fixed_E_polarization_vector=(1, 0, 0), wave_character=fx.WaveCharacter(wavelength=WL)))
    for n, z in dets:
        objs.append(fx.PoyntingFluxDetector(name=n, grid_slice_tuple=((0, 3), (0, 3), (z, z + 1)), direction="+",
                                            reduce_volume=True))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cuda")
    _, out = fx.run_fdtd(arrays, objects, cfg)
    spp = round(WL / (C0 * cfg.time_step_duration))
    return {n: float(out.detector_states[n]["poynting_flux"][:, 0].double()[-10 * spp:].mean().cpu()) for n, _ in dets}


def test_lorentz_and_drude_half_spaces_on_the_gpu():
    """Fresnel transmission into a Lorentz half-space within 5% (test_dispersion.py:228-262);
    a Drude metal transmits below 0.05 and absorbs the Fresnel fraction 1 - R within 10%; a
    plane source inside a uniform Lorentz medium injects its impedance: backward / forward
    flux below 2% (test_dispersion.py:329-360)."""
    s0 = _gpu_flux(None, dets=(("t", 140), ("n", 60)))
    lor = _gpu_flux(fx.Material(permittivity=1.0, dispersion=_lorentz()))
    t_lor = _fresnel_t(1.0 + _lorentz().susceptibility(OMEGA))
    dru = _gpu_flux(fx.Material(permittivity=1.0, dispersion=_drude()), dets=(("t", 140), ("n", 60)))
    t_dru = _fresnel_t(1.0 + _drude().susceptibility(OMEGA))
    emb = _gpu_flux(fx.Material(permittivity=1.0, dispersion=_lorentz()), half=False, src_z=60,
                    dets=(("fwd", 90), ("bwd", 30)))
    log_result("dispersion_physics_gpu", T_lorentz=lor["t"] / s0["t"], T_lorentz_ref=t_lor,
               absorbed_drude=dru["n"] / s0["n"], T_drude_ref=t_dru, embedded_bwd_over_fwd=abs(emb["bwd"]) / emb["fwd"])
    assert s0["t"] > 0 and abs(lor["t"] / s0["t"] - t_lor) / t_lor < 0.05
    assert abs(dru["t"] / s0["t"] - t_dru) < 0.05 and abs(dru["n"] / s0["n"] - t_dru) / t_dru < 0.10
    assert emb["fwd"] > 0 and abs(emb["bwd"]) / emb["fwd"] < 0.02


def test_dispersive_reverse_is_refused():
    """The ADE polarisation has no reverse step: the native reverse returns FDTD_EINVAL."""
    objs = [fx.SimulationVolume(shape=(6, 6, 6)),
            fx.UniformMaterialObject(name="m", grid_slice_tuple=((0, 6), (0, 6), (0, 6)),
                                     material=fx.Material(dispersion=_lorentz()))]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, fx.SimulationConfig(time=4e-16, grid=fx.UniformGrid(25e-9)),
                                                  device="cuda")
    scene = Scene(objects, arrays, cfg)
    scene.forward(arrays, 0, 2, graph=False)
    with pytest.raises(N.NativeError, match="dispersive"):
        scene.reverse(arrays, 2, 2)
    scene.close()


@pytest.mark.parametrize("segments", [1, 4])
def test_dispersive_checkpointed_gradient(segments):
    """The reference's gradient method for dispersive materials, GradientConfig(method=
    "checkpointed"): d|phasor|^2 / d inv_eps through the stored-state backward pass with the ADE
    step transposed (k_ade_T), against autograd through the oracle's forward run over the whole
    grid (float32 oracle asserted: both store the ADE coefficients in float32; float64
    reported)."""
    dx = 25e-9
    nx, ny, nz = 6, 6, 70
    wc = fx.WaveCharacter(wavelength=WL)
    pulse = fx.GaussianPulseProfile(spectral_width=fx.WaveCharacter(frequency=0.2 * C0 / WL), center_wave=wc)
    gc = fx.GradientConfig(method="checkpointed", num_checkpoints=segments)
    cfg = fx.SimulationConfig(time=160 * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx), gradient_config=gc)
    vol = fx.SimulationVolume(shape=(nx, ny, nz))
    bc = fx.BoundaryConfig.from_uniform_bound(8, override_types={"min_x": "periodic", "max_x": "periodic",
                                                                 "min_y": "periodic", "max_y": "periodic"})
    poles = _lorentz().poles + (fx.DrudePole(plasma_frequency=1.5 * OMEGA, damping=0.05 * OMEGA),)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs += [
        fx.UniformMaterialObject(name="slab", grid_slice_tuple=((0, nx), (0, ny), (30, 50)), material=fx.Material(
            permittivity=1.5, electric_conductivity=2e3, dispersion=fx.DispersionModel(poles=poles))),
        fx.UniformPlaneSource(name="pl", grid_slice_tuple=((0, nx), (0, ny), (15, 16)), direction="+",
                              fixed_E_polarization_vector=(1, 0, 0), wave_character=wc, temporal_profile=pulse),
        fx.PhasorDetector(name="ph", grid_slice_tuple=((0, nx), (0, ny), (25, 55)), wave_characters=(wc,)),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cuda")
    ie = arrays.inv_permittivities.clone().requires_grad_(True)
    _, out = fx.run_fdtd(arrays.aset("inv_permittivities", ie), objects, cfg)
    (out.detector_states["ph"]["phasor"].abs() ** 2).sum().backward()
    g_gpu = ie.grad.detach().cpu()
    res = {}
    for dt in (torch.float32, torch.float64):
        sc = O.OracleScene(objects, arrays, cfg, dt)
        res[dt] = O.autograd_gradient(sc, lambda det: (det["ph"]["phasor"].abs() ** 2).sum(), cfg.time_steps_total)
    e32 = float(torch.linalg.vector_norm(g_gpu.double() - res[torch.float32].double().cpu())
                / torch.linalg.vector_norm(res[torch.float32].double()))
    e64 = float(torch.linalg.vector_norm(g_gpu.double() - res[torch.float64].double().cpu())
                / torch.linalg.vector_norm(res[torch.float64].double()))
    log_result(f"dispersion_checkpointed_gradient_{segments}", grad_rel_l2_vs_fp32_autograd=e32,
               grad_rel_l2_vs_fp64_autograd=e64)
    assert torch.linalg.vector_norm(res[torch.float64]).item() > 0 and e32 <= 1e-3, (e32, e64)
