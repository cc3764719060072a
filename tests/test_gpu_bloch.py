"""Bloch boundaries with a non-zero vector on the GPU: complex fields against the oracle.

The kernels carry a complex field as its real and imaginary parts (planar) and update them
part by part; only a neighbour wrapped across a Bloch axis mixes the two, multiplied by the
phase exp(i k L) (the '+' ghost layer) or its conjugate (the '-' one)
(fdtdx/fdtd/update.py:92-136, fdtdx/objects/boundaries/bloch.py:59-94).  Sources drive the
real parts; phasor detectors take the complex sample, field detectors its real part, flux
detectors Re(E x conj H) and energy detectors |E|^2 and |H|^2.  Tolerance: relative L2 <=
1e-4 against the float32 oracle (float64 reported); gradients 1e-3 (the reversible adjoint
re-rounds 2T steps).
"""

from __future__ import annotations

import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300.engine import Scene
from oracle import fdtd_oracle as O
from tests.helpers import compare_states, log_result, rel_l2
from tests.test_gpu_adjoint import _inner, _to_cuda

pytestmark = pytest.mark.gpu
TOL = 1e-4
C0 = 299792458.0
FACES = ("min_x", "max_x", "min_y", "max_y", "min_z", "max_z")


def _cfg(steps, dx=50e-9, record=False):
    return fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx),
                               gradient_config=fx.GradientConfig(recorder=fx.Recorder()) if record else None)


def _place(types, kv, shape, steps, extra=(), record=False, pml=4, dx=50e-9, **pml_kw):
    cfg = _cfg(steps, dx, record)
    vol = fx.SimulationVolume(shape=shape)
    bc = fx.BoundaryConfig.from_uniform_bound(pml, override_types=types, bloch_vector=kv, **pml_kw)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values()) + list(extra)
    return fx.place_objects(objs, cfg, device="cuda")


def _seeded(shape, seed=42):
    g = torch.Generator().manual_seed(seed)

    def rnd():
        return torch.complex(torch.randn((3, *shape), generator=g), torch.randn((3, *shape), generator=g)) * 1e-3

    return rnd(), rnd()


@pytest.mark.parametrize("mixed", [False, True])
def test_bloch_seeded_steps_match_oracle(mixed):
    """Seeded complex fields, 12 steps: Bloch on every face with a vector along all three axes,
    or Bloch x and y with CPML z (kappa != 1) and a lossy block; E, H and psi."""
    types = {f: "bloch" for f in (FACES[:4] if mixed else FACES)}
    kv = (1.2e6, -0.8e6, 0.0) if mixed else (1.3e6, -0.7e6, 2.1e6)
    blk = fx.UniformMaterialObject(name="blk", grid_slice_tuple=((3, 9), (2, 8), (4, 12)),
                                   material=fx.Material(permittivity=(4.0, 3.0, 2.5), electric_conductivity=2e4))
    objects, arrays, _, cfg, _ = _place(types, kv, (12, 11, 16), 12, extra=(blk,), kappa_end=1.5)
    assert arrays.fields.E.dtype == torch.complex64
    E0, H0 = _seeded((12, 11, 16))
    sc32 = O.OracleScene(objects, arrays, cfg, torch.float32)
    sc64 = O.OracleScene(objects, arrays, cfg, torch.float64)
    E0 = O._walls(sc64, E0.to(torch.complex128), sc64.pec).to(torch.complex64)
    work = arrays.aset("fields->E", E0.cuda().contiguous()).aset("fields->H", H0.cuda().contiguous())
    scene = Scene(objects, work, cfg)
    assert scene.complex_fields
    scene.forward(work, 0, 12, graph=False)
    scene.status()
    torch.cuda.synchronize()
    refs = []
    for sc in (sc32, sc64):
        st = sc.init_state()
        st.E, st.H = E0.to(sc.field_dtype), H0.to(sc.field_dtype)
        refs.append(O.run(sc, 12, state=st))
    compare_states(f"bloch_seeded_{'mixed' if mixed else 'all'}", work, refs[0], refs[1], TOL)
    for p in sc32.pmls:
        for q in range(2):
            assert rel_l2(work.fields.psi_E[p.name][q], refs[0].psi_E[p.name][q]) <= 5 * TOL
            assert rel_l2(work.fields.psi_H[p.name][q], refs[0].psi_H[p.name][q]) <= 5 * TOL
    assert (mixed and sc32.pmls) or not mixed
    scene.close()


def test_bloch_sources_and_every_detector():
    """Bloch x (periodic y, CPML z): a tilted plane source and a dipole, and every detector kind
    (phasor volume and reduced, field plane and reduced, flux reduced and per cell, energy),
    exact and plain interpolation, through run_fdtd with a CUDA graph."""
    wc = fx.WaveCharacter(wavelength=1.0e-6)
    nx, ny, nz = 16, 6, 40
    R = ((0, nx), (0, ny), (14, 26))
    extra = (
        fx.UniformMaterialObject(name="d", grid_slice_tuple=((0, nx), (0, ny), (24, 34)),
                                 material=fx.Material(permittivity=2.25)),
        fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, nx), (0, ny), (10, 11)), direction="+",
                              fixed_E_polarization_vector=(0, 1, 0), azimuth_angle=25.0, wave_character=wc),
        fx.PointDipoleSource(name="dip", grid_slice_tuple=((5, 6), (2, 3), (18, 19)), polarization=2,
                             wave_character=wc),
        fx.PhasorDetector(name="ph", grid_slice_tuple=R, wave_characters=(wc,)),
        fx.PhasorDetector(name="ph_red", grid_slice_tuple=R, wave_characters=(wc,), components=("Ey", "Hx"),
                          reduce_volume=True),
        fx.FieldDetector(name="f_plane", grid_slice_tuple=((0, nx), (0, ny), (20, 21)), components=("Ex", "Ey", "Hz")),
        fx.FieldDetector(name="f_red", grid_slice_tuple=R, reduce_volume=True, exact_interpolation=False),
        fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((0, nx), (0, ny), (30, 31)), direction="+"),
        fx.PoyntingFluxDetector(name="flux_cells", grid_slice_tuple=((0, nx), (0, ny), (16, 17)), direction="-",
                                keep_all_components=True, reduce_volume=False),
        fx.EnergyDetector(name="en", grid_slice_tuple=R, reduce_volume=True),
    )
    kx = 2 * math.pi / 1.0e-6 * math.sin(math.radians(25.0))
    objects, arrays, _, cfg, _ = _place({f: "bloch" for f in FACES[:2]} | {f: "periodic" for f in FACES[2:4]},
                                        (kx, 0.0, 0.0), (nx, ny, nz), 160, extra=extra, pml=6)
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    res = []
    for dt in (torch.float32, torch.float64):
        sc = O.OracleScene(objects, arrays, cfg, dt)
        assert sc.field_dtype.is_complex
        res.append(O.run(sc))
    assert torch.linalg.vector_norm(res[1].det["ph"]["phasor"]).item() > 0
    compare_states("bloch_sources_detectors", out, res[0], res[1], TOL)


def test_bloch_reverse_restores_with_recording():
    """Forward 40 steps recording the CPML interfaces, then 40 reverse steps: the interior
    returns to the seeded state, and the kernels' reverse agrees with the oracle's."""
    kv = (1.0e6, 0.6e6, 0.0)
    objects, _, _, cfg, _ = _place({f: "bloch" for f in FACES[:4]}, kv, (10, 9, 24), 40, record=True, pml=5)
    from fdtdx_gb300.initialization import init_arrays

    arrays = init_arrays(objects, cfg, device="cuda")
    assert arrays.recording_state.data["interfaces"].dtype == torch.complex64
    E0, H0 = _seeded((10, 9, 24), seed=7)
    work = arrays.aset("fields->E", E0.cuda()).aset("fields->H", H0.cuda())
    scene = Scene(objects, work, cfg, record_interfaces=True)
    scene.forward(work, 0, 40)
    scene.reverse(work, 40, 40)
    scene.status()
    torch.cuda.synchronize()
    inner = (slice(None), slice(None), slice(None), slice(6, -6))
    eE = rel_l2(work.fields.E[inner], E0[inner])
    eH = rel_l2(work.fields.H[inner], H0[inner])
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    st = sc.init_state()
    st.E, st.H = E0.to(torch.complex128), H0.to(torch.complex128)
    st = O.run(sc, 40, record_boundaries=True, state=st)
    for _ in range(40):
        st = O.backward(sc, st)
    eo = rel_l2(work.fields.E[inner], st.E[inner])
    log_result("bloch_reverse_roundtrip", rel_l2_E=eE, rel_l2_H=eH, vs_oracle_reverse=eo)
    assert eE < 1e-3 and eH < 1e-3 and eo < 1e-3
    scene.close()


def test_bloch_oblique_fresnel_te():
    """The reference's oblique-incidence check on the GPU: a 30-degree TE plane wave in a 20-cell
    Bloch cell (k_x = k0 sin 30 degrees) crossing a vacuum / eps_r = 4 interface transmits the
    Fresnel T within 5% (tests/simulation/physics/boundaries/test_bloch_oblique.py)."""
    wl, dx, nx, nz = 1e-6, 25e-9, 20, 160
    theta = math.radians(30.0)
    k_x = 2 * math.pi / wl * math.sin(theta)
    out = []
    for diel in (False, True):
        cfg = fx.SimulationConfig(time=120e-15, grid=fx.UniformGrid(dx))
        vol = fx.SimulationVolume(shape=(nx, 3, nz))
        bc = fx.BoundaryConfig.from_uniform_bound(10, override_types={"min_x": "bloch", "max_x": "bloch",
                                                                      "min_y": "periodic", "max_y": "periodic"},
                                                  bloch_vector=(k_x, 0.0, 0.0))
        objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
        if diel:
            objs.append(fx.UniformMaterialObject(name="d", grid_slice_tuple=((0, nx), (0, 3), (80, nz)),
                                                 material=fx.Material(permittivity=4.0)))
        objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, nx), (0, 3), (14, 15)), direction="+",
                                          fixed_E_polarization_vector=(0, 1, 0), azimuth_angle=30.0,
                                          wave_character=fx.WaveCharacter(wavelength=wl)))
        objs.append(fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((0, nx), (0, 3), (120, 121)), direction="+",
                                            reduce_volume=True))
        objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cuda")
        _, res = fx.run_fdtd(arrays, objects, cfg)
        spp = round(wl / (C0 * cfg.time_step_duration))
        out.append(float(res.detector_states["flux"]["poynting_flux"][:, 0].double()[-10 * spp:].mean()))
    s0, s1 = out
    tt = math.asin(math.sin(theta) / 2.0)
    t_ref = (2.0 * math.cos(tt)) / math.cos(theta) * (2.0 * math.cos(theta) / (math.cos(theta) + 2.0 * math.cos(tt))) ** 2
    log_result("bloch_oblique_fresnel_gpu", T=s1 / s0, T_ref=t_ref)
    assert s0 > 0 and abs(s1 / s0 - t_ref) / t_ref < 0.05, (s1 / s0, t_ref)


def _bloch_gradient_scene(steps, ckpt=0):
    """Bloch x and y (a vector along both), CPML z with kappa != 1, an anisotropic lossy block,
    a dipole and a plane source, and every detector kind; recorded for the reversible gradient."""
    dx = 40e-9
    nx, ny, nz = 14, 12, 30
    cfg = fx.SimulationConfig(time=steps * 0.99 / math.sqrt(3) * dx / C0, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder(),
                                                                num_checkpoints_reversible=ckpt))
    vol = fx.SimulationVolume(shape=(nx, ny, nz))
    bc = fx.BoundaryConfig.from_uniform_bound(5, override_types={f: "bloch" for f in FACES[:4]},
                                              bloch_vector=(1.1e6, -0.6e6, 0.0), kappa_end=1.5)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    wc = fx.WaveCharacter(wavelength=1.0e-6)
    R = ((2, 12), (1, 11), (11, 20))
    objs += [
        fx.UniformMaterialObject(name="blk", grid_slice_tuple=((3, 10), (2, 9), (12, 19)),
                                 material=fx.Material(permittivity=(2.0, 4.0, 3.0), electric_conductivity=2e4)),
        fx.UniformPlaneSource(name="src", grid_slice_tuple=((0, nx), (0, ny), (8, 9)), direction="+",
                              fixed_E_polarization_vector=(0, 1, 0), wave_character=wc),
        fx.PointDipoleSource(name="dip", grid_slice_tuple=((6, 7), (5, 6), (15, 16)), polarization=0,
                             wave_character=wc),
        fx.PhasorDetector(name="ph", grid_slice_tuple=R, wave_characters=(wc,)),
        fx.PhasorDetector(name="ph_red", grid_slice_tuple=R, wave_characters=(wc,), components=("Ex", "Hz"),
                          reduce_volume=True),
        fx.FieldDetector(name="f_plane", grid_slice_tuple=((0, nx), (0, ny), (16, 17)), components=("Ey", "Hx")),
        fx.FieldDetector(name="f_red", grid_slice_tuple=R, reduce_volume=True, exact_interpolation=False),
        fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((0, nx), (0, ny), (21, 22)), direction="+"),
        fx.PoyntingFluxDetector(name="flux_all", grid_slice_tuple=((4, 9), (3, 8), (13, 15)), direction="-",
                                keep_all_components=True, reduce_volume=False),
        fx.EnergyDetector(name="en", grid_slice_tuple=R, reduce_volume=True),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


def _random_cotangents(arrays, seed):
    g = torch.Generator().manual_seed(seed)

    def rnd(v):
        if v.is_complex():
            return torch.complex(torch.randn(v.shape, generator=g), torch.randn(v.shape, generator=g))
        return torch.randn(v.shape, generator=g)

    cots = {(dn, k): rnd(v) for dn, st in arrays.detector_states.items() for k, v in st.items()}
    return cots, rnd(arrays.fields.E), rnd(arrays.fields.H)


@pytest.mark.parametrize("ckpt", [0, 2])
def test_bloch_reversible_gradient_every_detector(ckpt):
    """d <cot, outputs> / d inv_eps of a Bloch scene through reversible_fdtd against the oracle's
    restatement of the custom VJP (fdtdx/fdtd/fdtd.py:215-333) on complex fields: seeded complex
    cotangents on E, H and every detector state; one slice and three (checkpoint resets)."""
    objects, arrays, cfg = _bloch_gradient_scene(60, ckpt)
    assert arrays.fields.E.dtype == torch.complex64
    cots, cE, cH = _random_cotangents(arrays, 11)

    def loss(out):
        tot = _inner(cE.cuda(), out.fields.E) + _inner(cH.cuda(), out.fields.H)
        for (dn, k), c in cots.items():
            v = out.detector_states[dn][k]
            tot = tot + _inner(c.cuda().to(v.dtype), v)
        return tot

    ga = _to_cuda(objects, arrays)
    ie = ga.inv_permittivities.clone().requires_grad_(True)
    _, out = fx.reversible_fdtd(ga.aset("inv_permittivities", ie), objects, cfg)
    loss(out).backward()
    torch.cuda.synchronize()
    g_gpu = ie.grad.detach().cpu()
    res = {}
    for dt in (torch.float32, torch.float64):
        sc = O.OracleScene(objects, arrays, cfg, dt)
        cdt = sc.field_dtype
        f = O.run(sc, cfg.time_steps_total, record_boundaries=True)
        cd = {}
        for (dn, k), c in cots.items():
            cd.setdefault(dn, {})[k] = c.to(cdt if c.is_complex() else dt)
        res[dt] = O.reversible_gradient(sc, f, cd, cE.to(cdt), cH.to(cdt))
    # checkpoint resets change the gradient inside the CPML by design (psi is frozen in the
    # reconstruction); outside it the sliced and the single-slice gradients are the same
    sl = (slice(None), slice(None), slice(None), slice(6, -6)) if ckpt else (slice(None),) * 4
    e32, e64 = rel_l2(g_gpu[sl], res[torch.float32][sl]), rel_l2(g_gpu[sl], res[torch.float64][sl])
    log_result(f"bloch_gradient_ckpt{ckpt}", grad_rel_l2_vs_fp32=e32, grad_rel_l2_vs_fp64=e64,
               fp32_oracle_vs_fp64=rel_l2(res[torch.float32], res[torch.float64]))
    assert torch.linalg.vector_norm(res[torch.float64]).item() > 0
    assert e32 <= 1e-3, (e32, e64)


def test_bloch_gradient_matches_autograd_of_the_complex_run():
    """The Bloch gradient of a phasor objective against float64 autograd through the oracle's
    complex forward run (a check independent of the reversible restatement), away from the
    CPML slabs where the reconstruction is not a time reversal."""
    objects, arrays, cfg = _bloch_gradient_scene(50)
    ga = _to_cuda(objects, arrays)
    ie = ga.inv_permittivities.clone().requires_grad_(True)
    _, out = fx.reversible_fdtd(ga.aset("inv_permittivities", ie), objects, cfg)
    (out.detector_states["ph"]["phasor"].abs() ** 2).sum().backward()
    g_gpu = ie.grad.detach().cpu()
    sc = O.OracleScene(objects, arrays, cfg, torch.float64)
    g_ad = O.autograd_gradient(sc, lambda det: (det["ph"]["phasor"].abs() ** 2).sum(), cfg.time_steps_total)
    inner = (slice(None), slice(None), slice(None), slice(6, -6))
    e = rel_l2(g_gpu[inner], g_ad[inner].float())
    log_result("bloch_gradient_vs_autograd", rel_l2=e)
    assert torch.linalg.vector_norm(g_ad).item() > 0 and e <= 1e-3, e
