"""Pins of the oracle's reversible gradient (CPU, float64).

The reference's strongest gradient check is reversible vs checkpointed on a periodic
lossy slab with a dipole (tests/simulation/fdtd/test_fdtd.py:394-463, rel < 1e-5 in
float64, loss sum(E^2)).  The oracle replays it: its restatement of the custom VJP
(reverse reconstruction + per-step VJP, T+1 steps) against plain autograd through the
forward run.  With CPML the reconstruction is exact in the interior only (interfaces are
re-imposed, the absorbing layer is not reversible), so there the check covers the
interior cells.
"""

import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import scenes
from oracle import fdtd_oracle as O

C0 = 299792458.0


def _periodic_lossy_slab(n=8, dx=50e-9, time=40e-15):
    cfg = fx.SimulationConfig(time=time, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    vol = fx.SimulationVolume(shape=(n, n, n))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(4, "periodic"),
                                                        vol).values())
    objs.append(fx.UniformMaterialObject(name="slab", grid_slice_tuple=((0, n), (0, n), (n // 4, n // 4 + n // 2)),
                                         material=fx.Material(permittivity=2.0, electric_conductivity=1e2)))
    objs.append(fx.PointDipoleSource(name="dip", grid_slice_tuple=((n // 2, n // 2 + 1),) * 3, polarization=0,
                                     wave_character=fx.WaveCharacter(frequency=C0 / 800e-9)))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


def _autograd_fields_loss(sc, T):
    ie = sc.inv_eps.clone().requires_grad_(True)
    st = sc.init_state()
    for _ in range(T):
        st = O.forward(sc, st, inv_eps=ie)
    loss = (st.E**2).sum()
    (g,) = torch.autograd.grad(loss, [ie])
    return loss.detach(), g


def test_reversible_matches_autograd_periodic_lossy_slab():
    objects, arrays, cfg = _periodic_lossy_slab()
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total
    assert 400 <= T <= 450
    loss_chk, g_chk = _autograd_fields_loss(sc, T)
    final = O.run(sc, T, record_boundaries=True)
    g_rev = O.reversible_gradient(sc, final, {}, cot_E=2 * final.E)
    assert torch.isclose((final.E**2).sum(), loss_chk, rtol=1e-9, atol=1e-12)
    max_abs = (g_rev.abs() + g_chk.abs()).max().item()
    rel = (g_rev - g_chk).abs().max().item() / (max_abs + 1e-30)
    assert max_abs > 0 and rel < 1e-5, rel


def _pml_scene(n=(18, 16, 16), pml=4, steps=70):
    dx = 50e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    vol = fx.SimulationVolume(shape=n)
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(pml), vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((7, 11), (6, 10), (6, 10)),
                                         material=fx.Material(permittivity=4.0)))
    objs.append(fx.PointDipoleSource(name="dip", grid_slice_tuple=((6, 7), (8, 9), (8, 9)), polarization=2,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    wc = fx.WaveCharacter(wavelength=1.55e-6)
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((12, 13), (5, 11), (5, 11)), wave_characters=(wc,),
                                  components=("Ex", "Ey", "Ez"), scaling_mode="pulse"))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


def test_reversible_matches_autograd_interior_with_cpml():
    objects, arrays, cfg = _pml_scene()
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total

    def loss_fn(det):
        return (det["ph"]["phasor"].abs() ** 2).sum()

    g_chk = O.autograd_gradient(sc, loss_fn, T)
    final = O.run(sc, T, record_boundaries=True)
    ph = final.det["ph"]["phasor"]
    g_rev = O.reversible_gradient(sc, final, {"ph": {"phasor": 2 * ph}})
    interior = (slice(None), slice(5, -5), slice(5, -5), slice(5, -5))
    a, b = g_rev[interior], g_chk[interior]
    rel = (a - b).abs().max().item() / (b.abs().max().item() + 1e-30)
    assert b.abs().max().item() > 0 and rel < 1e-6, rel


def test_slice_boundaries_match_reference_rule():
    """fdtd.py:20-36: round(i * T / k); every slice non-empty when k <= T."""
    from fdtdx_gb300.adjoint import reversible_slice_boundaries

    assert reversible_slice_boundaries(10, 1) == [0, 10]
    assert reversible_slice_boundaries(10, 3) == [0, 3, 7, 10]
    b = reversible_slice_boundaries(7, 7)
    assert b == list(range(8))
    with pytest.raises(Exception):
        cfg = fx.SimulationConfig(time=5 * 1e-17, grid=fx.UniformGrid(50e-9),
                                  gradient_config=fx.GradientConfig(recorder=fx.Recorder(),
                                                                    num_checkpoints_reversible=-1))
        del cfg


def _periodic_magnetic_slab(n=8, dx=50e-9, time=30e-15, permeability=1.5):
    cfg = fx.SimulationConfig(time=time, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    vol = fx.SimulationVolume(shape=(n, n, n))
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(4, "periodic"),
                                                        vol).values())
    objs.append(fx.UniformMaterialObject(
        name="slab", grid_slice_tuple=((0, n), (0, n), (n // 4, n // 4 + n // 2)),
        material=fx.Material(permittivity=2.0, permeability=permeability, electric_conductivity=1e2,
                             magnetic_conductivity=3e7)))
    objs.append(fx.PointDipoleSource(name="dip", grid_slice_tuple=((n // 2, n // 2 + 1),) * 3, polarization=0,
                                     wave_character=fx.WaveCharacter(frequency=C0 / 800e-9)))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


@pytest.mark.parametrize("permeability", [1.5, (1.5, 1.2, 2.0)])
def test_reversible_inv_mu_matches_autograd_periodic_magnetic_slab(permeability):
    """The reference's custom VJP returns d/d inv_permeabilities too (fdtd.py:331): the
    restatement against autograd through the forward run, loss sum(E^2) + sum(H^2)."""
    objects, arrays, cfg = _periodic_magnetic_slab(permeability=permeability)
    assert isinstance(arrays.inv_permeabilities, torch.Tensor)
    assert arrays.inv_permeabilities.shape[0] == (1 if isinstance(permeability, float) else 3)
    assert arrays.magnetic_conductivity is not None
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total
    ie = sc.inv_eps.clone().requires_grad_(True)
    im = sc.inv_mu.clone().requires_grad_(True)
    st = sc.init_state()
    for _ in range(T):
        st = O.forward(sc, st, inv_eps=ie, inv_mu=im)
    loss = (st.E**2).sum() + (st.H**2).sum()
    ge_chk, gm_chk = torch.autograd.grad(loss, [ie, im])
    final = O.run(sc, T, record_boundaries=True)
    ge, gm = O.reversible_gradient(sc, final, {}, cot_E=2 * final.E, cot_H=2 * final.H, with_mu=True)
    for a, b in ((ge, ge_chk), (gm, gm_chk)):
        scale = (a.abs() + b.abs()).max().item()
        assert scale > 0 and (a - b).abs().max().item() / scale < 1e-5


def _pml_magnetic_scene(n=(18, 16, 16), pml=4, steps=60):
    dx = 50e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    vol = fx.SimulationVolume(shape=n)
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(pml), vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((7, 11), (6, 10), (6, 10)),
                                         material=fx.Material(permittivity=3.0, permeability=1.8)))
    objs.append(fx.PointDipoleSource(name="dip", grid_slice_tuple=((6, 7), (8, 9), (8, 9)), polarization=2,
                                     wave_character=fx.WaveCharacter(wavelength=1.55e-6),
                                     temporal_profile=scenes.pulse_5fs()))
    wc = fx.WaveCharacter(wavelength=1.55e-6)
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((12, 13), (5, 11), (5, 11)), wave_characters=(wc,),
                                  components=("Ex", "Hy", "Hz"), scaling_mode="pulse"))
    objs.append(fx.EnergyDetector(name="en", grid_slice_tuple=((8, 10), (7, 9), (7, 9)), as_slices=False,
                                  reduce_volume=True))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


def test_reversible_inv_mu_matches_autograd_interior_with_cpml():
    """Phasor (E and H components) and energy objective: the inv_mu cotangent of the
    restatement agrees with autograd in the interior, where the reconstruction is exact."""
    objects, arrays, cfg = _pml_magnetic_scene()
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total

    def loss_fn(det):
        return (det["ph"]["phasor"].abs() ** 2).sum() + 1e3 * det["en"]["energy"].sum()

    g_chk = O.autograd_gradient(sc, loss_fn, T, wrt="mu")
    final = O.run(sc, T, record_boundaries=True)
    ph = final.det["ph"]["phasor"]
    en = final.det["en"]["energy"]
    _, g_rev = O.reversible_gradient(sc, final, {"ph": {"phasor": 2 * ph}, "en": {"energy": 1e3 * torch.ones_like(en)}},
                                     with_mu=True)
    interior = (slice(None), slice(5, -5), slice(5, -5), slice(5, -5))
    a, b = g_rev[interior], g_chk[interior]
    rel = (a - b).abs().max().item() / (b.abs().max().item() + 1e-30)
    assert b.abs().max().item() > 0 and rel < 1e-6, rel
