"""Reversible-gradient parity of the GB300 adjoint against the oracle.

The GPU path (fdtd_adjoint through ``reversible_fdtd``'s autograd Function) is
compared with the oracle's restatement of the reference's custom VJP in float32
(asserted) and float64 (reported), and with central finite differences of the float64
oracle forward run.  Gradient tolerance: relative L2 <= 1e-3 against the float32
oracle (a float32 adjoint accumulates T+1 transposed steps and T reverse steps, each
re-rounded, so it carries more rounding than one forward run).
"""

import math

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import scenes
from oracle import fdtd_oracle as O
from tests.helpers import log_result, rel_l2

pytestmark = pytest.mark.gpu
GTOL = 1e-3
C0 = 299792458.0


def _to_cuda(objects, arrays):
    """The placed arrays moved to the GPU (placement ran on the CPU for the oracle)."""
    f = arrays.fields
    fields = fx.FieldState(
        E=f.E.cuda(), H=f.H.cuda(),
        psi_E={k: (a.cuda(), b.cuda()) for k, (a, b) in f.psi_E.items()},
        psi_H={k: (a.cuda(), b.cuda()) for k, (a, b) in f.psi_H.items()},
    )
    mu = arrays.inv_permeabilities
    rec = arrays.recording_state
    if rec is not None:
        rec = fx.RecordingState({k: v.cuda() for k, v in rec.data.items()}, {k: v.cuda() for k, v in rec.state.items()})
    return fx.ArrayContainer(
        fields=fields,
        inv_permittivities=arrays.inv_permittivities.cuda(),
        inv_permeabilities=mu.cuda() if isinstance(mu, torch.Tensor) else mu,
        detector_states={k: {k2: v2.cuda() for k2, v2 in v.items()} for k, v in arrays.detector_states.items()},
        recording_state=rec,
        electric_conductivity=None if arrays.electric_conductivity is None else arrays.electric_conductivity.cuda(),
        magnetic_conductivity=None if arrays.magnetic_conductivity is None else arrays.magnetic_conductivity.cuda(),
    )


def _gpu_grad(objects, arrays, cfg, cot_fn):
    """d <cot, outputs> / d inv_eps through the public reversible_fdtd."""
    ga = _to_cuda(objects, arrays)
    ie = ga.inv_permittivities.clone().requires_grad_(True)
    _, out = fx.reversible_fdtd(ga.aset("inv_permittivities", ie), objects, cfg)
    loss = cot_fn(out)
    loss.backward()
    torch.cuda.synchronize()
    return out, ie.grad.detach().cpu()


def _inner(cot, x):
    """<cot, x> whose torch gradient w.r.t. x is cot (complex: Re(conj(cot) x))."""
    if x.is_complex():
        return (cot.real * x.real + cot.imag * x.imag).sum()
    return (cot * x).sum()


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


def _check(name, g_gpu, sc32, sc64, final32, final64, cots32, cots64, cot_E=None, cot_H=None):
    g32 = O.reversible_gradient(sc32, final32, cots32,
                                None if cot_E is None else cot_E(final32), None if cot_H is None else cot_H(final32))
    g64 = O.reversible_gradient(sc64, final64, cots64,
                                None if cot_E is None else cot_E(final64), None if cot_H is None else cot_H(final64))
    e32, e64 = rel_l2(g_gpu, g32), rel_l2(g_gpu, g64)
    log_result(name, grad_rel_l2_vs_fp32=e32, grad_rel_l2_vs_fp64=e64, fp32_oracle_vs_fp64=rel_l2(g32, g64))
    assert torch.linalg.vector_norm(g64).item() > 0
    assert e32 <= GTOL, (name, e32, e64)
    return g32, g64


def test_adjoint_periodic_lossy_slab_fields_loss():
    """The reference's reversible-vs-checkpointed scene: loss sum(E^2) at the end of the run."""
    objects, arrays, cfg = _periodic_lossy_slab()
    _, g = _gpu_grad(objects, arrays, cfg, lambda out: (out.fields.E**2).sum())
    sc32, sc64 = O.OracleScene(objects, arrays, cfg, torch.float32), O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total
    f32, f64 = O.run(sc32, T, record_boundaries=True), O.run(sc64, T, record_boundaries=True)
    _check("adjoint_periodic_lossy", g, sc32, sc64, f32, f64, {}, {}, cot_E=lambda f: 2 * f.E)


def _cpml_phasor_scene(shape=(26, 24, 24), pml=5, steps=90, recorder=None):
    dx = 50e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=recorder or fx.Recorder()))
    vol = fx.SimulationVolume(shape=shape)
    objs = [vol] + list(fx.boundary_objects_from_config(fx.BoundaryConfig.from_uniform_bound(pml), vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((10, 16), (9, 15), (9, 15)),
                                         material=fx.Material(permittivity=4.0)))
    wc = fx.WaveCharacter(wavelength=1.55e-6)
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((pml + 1, pml + 2), (pml, shape[1] - pml),
                                                                    (pml, shape[2] - pml)),
                                      direction="+", fixed_E_polarization_vector=(0, 1, 0), wave_character=wc,
                                      temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((18, 19), (8, 16), (8, 16)), wave_characters=(wc,),
                                  components=("Ex", "Ey", "Ez"), scaling_mode="pulse"))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


def test_adjoint_cpml_plane_source_phasor_objective():
    """CPML on all faces, TFSF plane source, |phasor|^2 objective (the inverse-design form)."""
    objects, arrays, cfg = _cpml_phasor_scene()
    out, g = _gpu_grad(objects, arrays, cfg, lambda o: (o.detector_states["ph"]["phasor"].abs() ** 2).sum())
    sc32, sc64 = O.OracleScene(objects, arrays, cfg, torch.float32), O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total
    f32, f64 = O.run(sc32, T, record_boundaries=True), O.run(sc64, T, record_boundaries=True)
    _check("adjoint_cpml_phasor", g, sc32, sc64, f32, f64,
           {"ph": {"phasor": 2 * f32.det["ph"]["phasor"]}}, {"ph": {"phasor": 2 * f64.det["ph"]["phasor"]}})


@pytest.mark.parametrize("modules", [
    [fx.LinearReconstructEveryK(k=3)],
    [fx.LinearReconstructEveryK(k=4, start_recording_after=5), fx.DtypeConversion(torch.float16)],
])
def test_adjoint_recorder_time_filter(modules):
    """Interfaces stored every k-th step and interpolated in the reverse steps (the recording
    holds the filter's stored steps only), against the oracle with the same recorder."""
    objects, arrays, cfg = _cpml_phasor_scene(recorder=fx.Recorder(modules))
    assert arrays.recording_state.data["interfaces"].shape[0] == cfg.gradient_config.recorder.slots(
        cfg.time_steps_total) < cfg.time_steps_total
    out, g = _gpu_grad(objects, arrays, cfg, lambda o: (o.detector_states["ph"]["phasor"].abs() ** 2).sum())
    sc32, sc64 = O.OracleScene(objects, arrays, cfg, torch.float32), O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total
    f32, f64 = O.run(sc32, T, record_boundaries=True), O.run(sc64, T, record_boundaries=True)
    if any(isinstance(m, fx.DtypeConversion) for m in modules):
        # the stored planes are rounded to the storage dtype: so are the oracle's
        for f in (f32, f64):
            f.rec[:] = [{k: v.to(torch.float16).to(v.dtype) for k, v in r.items()} for r in f.rec]
    tol = "f16" if any(isinstance(m, fx.DtypeConversion) for m in modules) else "f32"
    g32 = O.reversible_gradient(sc32, f32, {"ph": {"phasor": 2 * f32.det["ph"]["phasor"]}})
    g64 = O.reversible_gradient(sc64, f64, {"ph": {"phasor": 2 * f64.det["ph"]["phasor"]}})
    e32, e64 = rel_l2(g, g32), rel_l2(g, g64)
    log_result(f"adjoint_time_filter_{tol}", grad_rel_l2_vs_fp32=e32, grad_rel_l2_vs_fp64=e64)
    assert e32 <= GTOL, (e32, e64)


def _all_detectors_scene(steps=70):
    dx = 25e-9
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    vol = fx.SimulationVolume(shape=(30, 28, 24), material=fx.Material(permittivity=2.1025))
    bc = fx.BoundaryConfig.from_uniform_bound(5, "pml", kappa_end=1.5)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(
        name="aniso", grid_slice_tuple=((9, 20), (8, 19), (8, 16)),
        material=fx.Material(permittivity=(2.0, 5.0, 9.0), electric_conductivity=(3e4, 1e4, 0.0))))
    wc = fx.WaveCharacter(wavelength=1.55e-6)
    objs.append(fx.GaussianPlaneSource(name="g", grid_slice_tuple=((7, 8), (7, 21), (6, 18)), direction="+",
                                       radius=5 * dx, fixed_E_polarization_vector=(0, 0, 1), wave_character=wc,
                                       temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PointDipoleSource(name="m", grid_slice_tuple=((14, 15), (12, 13), (11, 12)), polarization=1,
                                     source_type="magnetic", wave_character=wc, temporal_profile=scenes.pulse_5fs()))
    R = ((11, 19), (10, 18), (9, 15))
    objs += [
        fx.PhasorDetector(name="ph_all", grid_slice_tuple=R, wave_characters=(wc, fx.WaveCharacter(wavelength=1.3e-6))),
        fx.PhasorDetector(name="ph_red", grid_slice_tuple=R, wave_characters=(wc,), components=("Ey", "Hz"),
                          reduce_volume=True, scaling_mode="pulse", switch=fx.OnOffSwitch(interval=2)),
        fx.FieldDetector(name="f_plane", grid_slice_tuple=((0, 30), (0, 28), (12, 13)), components=("Ex", "Hy")),
        fx.FieldDetector(name="f_red", grid_slice_tuple=R, components=("Ez", "Hx"), reduce_volume=True,
                         exact_interpolation=False),
        fx.PoyntingFluxDetector(name="flux", grid_slice_tuple=((21, 22), (8, 20), (7, 17)), direction="+"),
        fx.PoyntingFluxDetector(name="flux_all", grid_slice_tuple=((13, 17), (11, 15), (10, 12)), direction="-",
                                keep_all_components=True, reduce_volume=False, exact_interpolation=False),
        fx.EnergyDetector(name="en", grid_slice_tuple=((10, 20), (9, 19), (8, 16)), reduce_volume=True),
        fx.EnergyDetector(name="en_vol", grid_slice_tuple=((12, 16), (12, 16), (10, 14)), reduce_volume=False),
    ]
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    return objects, arrays, cfg


def test_adjoint_all_detectors_random_cotangents():
    """Every detector kind (exact / non-exact, reduced / not), anisotropic lossy material, kappa != 1
    CPML, plane and magnetic sources; seeded random cotangents on E, H and every detector state."""
    objects, arrays, cfg = _all_detectors_scene()
    g = torch.Generator().manual_seed(7)
    cots = {}
    for dn, st in arrays.detector_states.items():
        for k, v in st.items():
            if v.is_complex():
                c = torch.complex(torch.randn(v.shape, generator=g), torch.randn(v.shape, generator=g))
            else:
                c = torch.randn(v.shape, generator=g)
            cots[(dn, k)] = c
    cE = torch.randn(arrays.fields.E.shape, generator=g)
    cH = torch.randn(arrays.fields.H.shape, generator=g)

    def loss(out):
        tot = _inner(cE.cuda(), out.fields.E) + _inner(cH.cuda(), out.fields.H)
        for (dn, k), c in cots.items():
            tot = tot + _inner(c.cuda().to(out.detector_states[dn][k].dtype), out.detector_states[dn][k])
        return tot

    _, gg = _gpu_grad(objects, arrays, cfg, loss)
    sc32, sc64 = O.OracleScene(objects, arrays, cfg, torch.float32), O.OracleScene(objects, arrays, cfg, torch.float64)
    T = cfg.time_steps_total
    f32, f64 = O.run(sc32, T, record_boundaries=True), O.run(sc64, T, record_boundaries=True)

    def cd(dtype):
        out = {}
        for (dn, k), c in cots.items():
            out.setdefault(dn, {})[k] = c.to(torch.complex128 if c.is_complex() and dtype == torch.float64 else
                                              torch.complex64 if c.is_complex() else dtype)
        return out

    _check("adjoint_all_detectors", gg, sc32, sc64, f32, f64, cd(torch.float32), cd(torch.float64),
           cot_E=lambda f: cE.to(f.E.dtype), cot_H=lambda f: cH.to(f.H.dtype))


def test_adjoint_sliced_checkpoints_agree():
    """num_checkpoints_reversible = 3 (reset at the slice boundaries) against the single slice and
    against float64 autograd.  Inside the CPML the reconstruction is not a time reversal (psi is
    frozen), so the reset changes the gradient there by design; outside it both are exact."""
    objects, arrays, cfg = _cpml_phasor_scene(steps=60)
    lossf = lambda o: (o.detector_states["ph"]["phasor"].abs() ** 2).sum()  # noqa: E731
    _, g1 = _gpu_grad(objects, arrays, cfg, lossf)
    gc = fx.GradientConfig(recorder=fx.Recorder(), num_checkpoints_reversible=3)
    cfg3 = fx.SimulationConfig(time=cfg.time, grid=cfg.grid, gradient_config=gc)
    _, g3 = _gpu_grad(objects, arrays, cfg3, lossf)
    sc64 = O.OracleScene(objects, arrays, cfg, torch.float64)
    gx = O.autograd_gradient(sc64, lambda det: (det["ph"]["phasor"].abs() ** 2).sum(), cfg.time_steps_total)
    inner = (slice(None), slice(6, -6), slice(6, -6), slice(6, -6))
    e13, e3x = rel_l2(g3[inner], g1[inner]), rel_l2(g3[inner], gx[inner])
    log_result("adjoint_sliced", rel_l2_interior_vs_single=e13, rel_l2_interior_vs_fp64_autograd=e3x)
    assert e13 <= 1e-4 and e3x <= GTOL, (e13, e3x)


def test_adjoint_params_chain_and_finite_differences():
    """Design parameters -> apply_params -> reversible_fdtd -> |phasor|^2; the parameter gradient
    against central finite differences (h = 1e-3) of the float64 oracle at 16 seeded voxels."""
    objects, arrays, params, cfg, _ = scenes.inverse_design(shape=(28, 28, 24), steps=400, design=(8, 8, 3),
                                                            plane=(6, 6), pml=5, device="cpu")
    p = params["design"].clone()
    ga = _to_cuda(objects, arrays)
    pg = p.cuda().requires_grad_(True)
    a2, _, _ = fx.apply_params(ga, objects, {"design": pg})
    _, out = fx.reversible_fdtd(a2, objects, cfg)
    loss = (out.detector_states["objective"]["phasor"].abs() ** 2).sum()
    loss.backward()
    grad = pg.grad.detach().cpu().double()

    def f64_loss(pv):
        a, _, _ = fx.apply_params(arrays, objects, {"design": pv})
        sc = O.OracleScene(objects, a, cfg, torch.float64)
        st = O.run(sc, cfg.time_steps_total)
        return (st.det["objective"]["phasor"].abs() ** 2).sum().item()

    rng = torch.Generator().manual_seed(3)
    flat = torch.randperm(p.numel(), generator=rng)[:16]
    h = 1e-3
    fd, ad = [], []
    for q in flat.tolist():
        pp, pm = p.clone().double(), p.clone().double()
        pp.view(-1)[q] += h
        pm.view(-1)[q] -= h
        fd.append((f64_loss(pp) - f64_loss(pm)) / (2 * h))
        ad.append(grad.view(-1)[q].item())
    fd, ad = torch.tensor(fd), torch.tensor(ad)
    e = rel_l2(ad, fd)
    log_result("adjoint_fd_16_voxels", rel_l2=e, fd=fd.tolist(), adjoint=ad.tolist())
    assert e <= 2e-2, (e, fd, ad)


def _gpu_grads_eps_mu(objects, arrays, cfg, cot_fn):
    """d <cot, outputs> / d (inv_eps, inv_mu) through the public reversible_fdtd."""
    ga = _to_cuda(objects, arrays)
    ie = ga.inv_permittivities.clone().requires_grad_(True)
    im = ga.inv_permeabilities.clone().requires_grad_(True)
    _, out = fx.reversible_fdtd(ga.aset("inv_permittivities", ie).aset("inv_permeabilities", im), objects, cfg)
    cot_fn(out).backward()
    torch.cuda.synchronize()
    return ie.grad.detach().cpu(), im.grad.detach().cpu()


def _check_eps_mu(name, ge, gm, objects, arrays, cfg, cots, cot_E=None, cot_H=None):
    T = cfg.time_steps_total
    res = {}
    for dt in (torch.float32, torch.float64):
        sc = O.OracleScene(objects, arrays, cfg, dt)
        f = O.run(sc, T, record_boundaries=True)
        res[dt] = O.reversible_gradient(sc, f, cots(f), None if cot_E is None else cot_E(f),
                                        None if cot_H is None else cot_H(f), with_mu=True)
    (e32, m32), (e64, m64) = res[torch.float32], res[torch.float64]
    err = dict(eps_vs_fp32=rel_l2(ge, e32), eps_vs_fp64=rel_l2(ge, e64), mu_vs_fp32=rel_l2(gm, m32),
               mu_vs_fp64=rel_l2(gm, m64), fp32_oracle_mu_vs_fp64=rel_l2(m32, m64))
    log_result(name, **err)
    assert torch.linalg.vector_norm(m64).item() > 0
    assert err["eps_vs_fp32"] <= GTOL and err["mu_vs_fp32"] <= GTOL, err


@pytest.mark.parametrize("permeability", [1.5, (1.5, 1.2, 2.0)])
def test_adjoint_inv_mu_periodic_magnetic_slab(permeability):
    """d/d inv_permeabilities (cot[6] of the reference's custom VJP, fdtd.py:331) with magnetic
    conductivity, isotropic (n_mu 1) and diagonal (n_mu 3); loss sum(E^2) + sum(H^2)."""
    n, dx = 8, 50e-9
    cfg = fx.SimulationConfig(time=30e-15, grid=fx.UniformGrid(dx),
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
    ge, gm = _gpu_grads_eps_mu(objects, arrays, cfg, lambda o: (o.fields.E**2).sum() + (o.fields.H**2).sum())
    _check_eps_mu(f"adjoint_inv_mu_periodic_n{arrays.inv_permeabilities.shape[0]}", ge, gm, objects, arrays, cfg,
                  lambda f: {}, cot_E=lambda f: 2 * f.E, cot_H=lambda f: 2 * f.H)


def test_adjoint_inv_mu_cpml_detectors():
    """inv_mu cotangent with CPML (kappa != 1) on all faces, a magnetic block, a TFSF plane source,
    a phasor detector on E and H components and an energy detector (its 1/inv_mu term)."""
    dx = 50e-9
    steps = 70
    dt = 0.99 / math.sqrt(3) * dx / C0
    cfg = fx.SimulationConfig(time=steps * dt, grid=fx.UniformGrid(dx),
                              gradient_config=fx.GradientConfig(recorder=fx.Recorder()))
    shape, pml = (26, 24, 24), 5
    vol = fx.SimulationVolume(shape=shape)
    bc = fx.BoundaryConfig.from_uniform_bound(pml, "pml", kappa_end=1.5)
    objs = [vol] + list(fx.boundary_objects_from_config(bc, vol).values())
    objs.append(fx.UniformMaterialObject(name="blk", grid_slice_tuple=((10, 16), (9, 15), (9, 15)),
                                         material=fx.Material(permittivity=3.0, permeability=(1.8, 1.3, 2.2))))
    wc = fx.WaveCharacter(wavelength=1.55e-6)
    objs.append(fx.UniformPlaneSource(name="src", grid_slice_tuple=((pml + 1, pml + 2), (pml, shape[1] - pml),
                                                                    (pml, shape[2] - pml)),
                                      direction="+", fixed_E_polarization_vector=(0, 1, 0), wave_character=wc,
                                      temporal_profile=scenes.pulse_5fs()))
    objs.append(fx.PhasorDetector(name="ph", grid_slice_tuple=((18, 19), (8, 16), (8, 16)), wave_characters=(wc,),
                                  components=("Ey", "Hx", "Hz"), scaling_mode="pulse"))
    objs.append(fx.EnergyDetector(name="en", grid_slice_tuple=((11, 15), (10, 14), (10, 14)), reduce_volume=True))
    objects, arrays, _, cfg, _ = fx.place_objects(objs, cfg, device="cpu")
    assert arrays.inv_permeabilities.shape[0] == 3
    w_en = 1e3

    def loss(o):
        return (o.detector_states["ph"]["phasor"].abs() ** 2).sum() + w_en * o.detector_states["en"]["energy"].sum()

    ge, gm = _gpu_grads_eps_mu(objects, arrays, cfg, loss)
    _check_eps_mu("adjoint_inv_mu_cpml", ge, gm, objects, arrays, cfg,
                  lambda f: {"ph": {"phasor": 2 * f.det["ph"]["phasor"]},
                             "en": {"energy": w_en * torch.ones_like(f.det["en"]["energy"])}})


def test_reversible_runs_release_device_memory_without_gc():
    """Repeated gradient runs (a new scene each time, as an optimisation loop or a stream of
    one-at-a-time jobs makes them) return every device tensor when their outputs are dropped,
    with the cycle collector off: no reference cycle keeps a run's state alive."""
    import gc

    gc.collect()
    gc.disable()
    try:
        base = None
        for _ in range(3):
            objects, arrays, cfg = _periodic_lossy_slab()
            ga = _to_cuda(objects, arrays)
            ie = ga.inv_permittivities.clone().requires_grad_(True)
            _, out = fx.reversible_fdtd(ga.aset("inv_permittivities", ie), objects, cfg)
            (out.fields.E ** 2).sum().backward()
            torch.cuda.synchronize()
            del out, ie, ga, arrays, objects
            _, res = fx.run_fdtd(*_to_cuda_run(_periodic_lossy_slab()))
            del res
            torch.cuda.synchronize()
            if base is None:
                base = torch.cuda.memory_allocated()  # after the first run: lazily built global state
            assert torch.cuda.memory_allocated() == base
    finally:
        gc.enable()


def _to_cuda_run(placed):
    objects, arrays, cfg = placed
    return _to_cuda(objects, arrays), objects, cfg
