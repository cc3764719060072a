"""The product's host setup (fdtdx_gb300.engine / objects) against the oracle's independent
restatement of the same reference code: CPML coefficients, plane-source profiles and Yee
time offsets, per-step source and detector tables, material painting."""

import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import engine, scenes
from oracle import fdtd_oracle as O


@pytest.mark.parametrize("direction,axis,L", [("-", 0, 10), ("+", 2, 6), ("-", 1, 8)])
@pytest.mark.parametrize("kappa", [1.0, 2.5])
def test_pml_coefficients_match_oracle(direction, axis, L, kappa):
    p = fx.PerfectlyMatchedLayer(axis=axis, direction=direction, kappa_end=kappa)
    st = [(0, 30)] * 3
    st[axis] = (0, L) if direction == "-" else (30 - L, 30)
    p.place_on_grid(tuple(st))
    dx, dt = 20e-9, 0.99 / math.sqrt(3) * 20e-9 / 299792458.0
    mine = p.coefficients(dx, dt)
    ref = O.pml_coefficients(p, dx, dt, torch.float64)
    for k in ("a_E", "b_E", "inv_kappa_E", "a_H", "b_H", "inv_kappa_H"):
        np.testing.assert_allclose(mine[k], ref[k].flatten().numpy(), rtol=2e-6, atol=1e-12, err_msg=k)


@pytest.mark.parametrize("kind,axis,direction", [("gauss", 0, "+"), ("gauss", 1, "-"), ("uniform", 2, "+")])
def test_plane_source_profiles_match_oracle(kind, axis, direction):
    cfg = fx.SimulationConfig(time=1e-14, grid=fx.UniformGrid(25e-9))
    vol = fx.SimulationVolume(shape=(20, 22, 24), material=fx.Material(permittivity=2.1025))
    st = [(3, 17), (4, 18), (5, 19)]
    st[axis] = (7, 8)
    common = dict(name="src", grid_slice_tuple=tuple(st), direction=direction,
                  wave_character=fx.WaveCharacter(wavelength=1.55e-6))
    if kind == "gauss":
        pol = [0.0, 0.0, 0.0]
        pol[(axis + 1) % 3] = 1.0
        src = fx.GaussianPlaneSource(radius=6 * 25e-9, fixed_E_polarization_vector=tuple(pol), **common)
    else:
        pol = [0.0, 0.0, 0.0]
        pol[(axis + 2) % 3] = 1.0
        src = fx.UniformPlaneSource(fixed_H_polarization_vector=tuple(pol), **common)
    blk = fx.UniformMaterialObject(name="blk", grid_slice_tuple=((0, 10), (0, 22), (0, 12)),
                                   material=fx.Material(permittivity=12.11))
    objects, arrays, _, cfg, _ = fx.place_objects([vol, blk, src], cfg, device="cpu")
    E, H, oE, oH = engine.plane_source_profiles(src, arrays, cfg)
    sc = O.OracleScene(objects, arrays, cfg, dtype=torch.float64)
    s = sc.sources[0]
    P = E.shape[1]
    for mine, ref in ((E, s.E_inc), (H, s.H_inc), (oE, s.off_E), (oH, s.off_H)):
        np.testing.assert_allclose(mine, ref.reshape(3, P).numpy(), rtol=1e-5, atol=1e-9)


def test_source_and_detector_tables():
    objects, arrays, _, cfg, _ = scenes.dipole_boxes(shape=(30, 30, 30), steps=40, n_boxes=3, pml=5, device="cpu")
    T = cfg.time_steps_total
    assert T == 40
    src = objects["dipole"]
    on, teff = engine.source_time_tables(src, cfg)
    assert on.all() and teff[0] == -1 and teff[-1] == T
    det = objects["ez_plane"]
    slot, w = engine.detector_tables(det, cfg)
    assert w is None and slot[0] == T - 1 and list(slot[1:T + 1]) == list(range(T)) and slot[T + 1] == T - 1
    # a switch that records every 3rd step
    d2 = fx.PhasorDetector(name="p", grid_slice_tuple=((1, 2), (1, 2), (1, 2)),
                           wave_characters=(fx.WaveCharacter(wavelength=1.55e-6),), switch=fx.OnOffSwitch(interval=3))
    slot, w = engine.detector_tables(d2, cfg)
    on_steps = [t for t in range(T) if t % 3 == 0]
    assert [t for t in range(T) if slot[t + 1] == 0] == on_steps
    expect = np.exp(1j * 2 * math.pi * 299792458.0 / 1.55e-6 * 3 * cfg.time_step_duration) * 2 / len(on_steps)
    assert np.allclose(w[4, 0, 0] + 1j * w[4, 0, 1], expect, rtol=1e-5)
    assert np.allclose(w[2, 0], 0.0)


def test_material_painting_in_placement_order():
    cfg = fx.SimulationConfig(time=1e-15, grid=fx.UniformGrid(50e-9))
    vol = fx.SimulationVolume(shape=(10, 10, 10), material=fx.Material(permittivity=2.0))
    a = fx.UniformMaterialObject(name="a", grid_slice_tuple=((0, 6), (0, 10), (0, 10)),
                                 material=fx.Material(permittivity=4.0), placement_order=1)
    b = fx.UniformMaterialObject(name="b", grid_slice_tuple=((4, 10), (0, 10), (0, 10)),
                                 material=fx.Material(permittivity=8.0, electric_conductivity=10.0), placement_order=0)
    _, arrays, _, _, _ = fx.place_objects([vol, a, b], cfg, device="cpu")
    ie = arrays.inv_permittivities[0, :, 0, 0]
    assert torch.allclose(ie, torch.tensor([0.25] * 6 + [0.125] * 4))
    assert arrays.inv_permeabilities == 1.0
    sig = arrays.electric_conductivity[0, :, 0, 0]
    assert torch.allclose(sig, torch.tensor([0.0] * 6 + [10.0 * 50e-9] * 4))


def test_reversible_fdtd_rejects_unsupported_material_inputs():
    """Gradients the reversible path does not take are refused before any device work: the
    gradient of a full 3x3 (9-component) permittivity, and a 0-d permeability tensor that asks
    for a gradient (a permeability gradient needs a (1 | 3, nx, ny, nz) array).  A full tensor
    itself is taken: the scene runs its tensor half-steps."""
    from fdtdx_gb300.engine import Scene

    objects, arrays, _, cfg, _ = scenes.dipole_boxes(shape=(12, 12, 12), steps=4, n_boxes=1, pml=3, device="cpu")
    inv9 = torch.zeros((9, 12, 12, 12))
    inv9[0] = inv9[4] = inv9[8] = 1.0
    full = arrays.aset("inv_permittivities", inv9.requires_grad_(True))
    with pytest.raises(NotImplementedError, match="3x3"):
        fx.reversible_fdtd(full, objects, cfg)
    mu0 = arrays.aset("inv_permeabilities", torch.tensor(1.0, requires_grad=True))
    with pytest.raises(NotImplementedError):
        fx.reversible_fdtd(mu0, objects, cfg)
    sc = Scene(objects, arrays.aset("inv_permittivities", inv9.detach()), cfg)
    assert sc.full_tensor and sc.desc.n_eps == 9
