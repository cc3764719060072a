"""Parity of every benchmark workload against the oracle, at the workload's own sizes.

Each of the five workloads the benchmark measures is run on the GPU and compared with the
float32 oracle (asserted, relative L2 <= 1e-4 on fields and detector states; 1e-3 on
gradients) and the float64 oracle (reported):

* dipole in 20 boxes, 100^3, 1000 steps: ``test_gpu_forward.py::test_dipole_boxes_full_size``;
* two-strip coupler, 400 x 400 x 200 at 20 nm: the first 40 steps of the 8000-step scene at
  full size (every detector state, including the 768 MB full-volume phasor), and a 120 x 120
  x 60 coupler over 1500 steps (the CW ramp and the steady state; the TMA core with the
  full-volume phasor staged through its pipeline);
* inverse design, 200 x 200 x 100, 3000 steps: the reversible gradient at full size against
  central finite differences of the GPU forward (at 16 seeded voxels and along a seeded
  direction over the whole design region), and a 64 x 64 x 40 copy of the scene against the
  oracle's restatement of the reference's custom VJP;
* 64 strips: the two smallest of the benchmark's seeded strips, batched, over their 2000 steps;
* served stream: one forward and one gradient job of the benchmark's seeded request stream,
  served in a mix, against the oracle.
"""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import scenes
from fdtdx_gb300.engine import Scene
from oracle import fdtd_oracle as O
from tests.helpers import compare_states, log_result, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4
GTOL = 1e-3


def _oracles(objects, arrays, cfg, steps=None, record=False):
    out = []
    for dt in (torch.float32, torch.float64):
        sc = O.OracleScene(objects, arrays, cfg, dt)
        out.append((sc, O.run(sc, steps, record_boundaries=record)))
    return out


def test_coupler_full_size_first_steps():
    """The benchmark's scene itself (400 x 400 x 200, 8000-step tables): its first 40 steps."""
    steps = 40
    objects, arrays, _, cfg, _ = scenes.coupler(steps=8000, device="cuda")
    work = arrays.reset()
    scene = Scene(objects, work, cfg)
    assert scene.uses_tma
    scene.forward(work, 0, steps)
    scene.status()
    torch.cuda.synchronize()
    scene.close()
    (_, r32), (_, r64) = _oracles(objects, arrays, cfg, steps)
    assert torch.linalg.vector_norm(r64.det["phasor"]["phasor"]).item() > 0
    compare_states("coupler_400x400x200_40_steps", work, r32, r64, TOL)


def test_coupler_scaled_long_run():
    """A 120 x 120 x 60 coupler for 1500 steps (CW ramp of four periods, then steady state):
    E, H, the full-volume phasor and both flux-plane phasors through run_fdtd."""
    objects, arrays, _, cfg, _ = scenes.coupler(shape=(120, 120, 60), steps=1500, scale=0.3, device="cuda")
    _, out = fx.run_fdtd(arrays, objects, cfg)
    torch.cuda.synchronize()
    from fdtdx_gb300.fdtd import get_scene

    assert get_scene(objects, out, cfg).uses_tma
    (_, r32), (_, r64) = _oracles(objects, arrays, cfg)
    res = compare_states("coupler_120x120x60_1500_steps", out, r32, r64, TOL)
    assert "phasor.phasor" in res and "flux1.phasor" in res
    for n in ("flux1", "flux2"):
        d = objects[n]
        g = d.compute_poynting_flux(out.detector_states[n], cfg.grid.spacing)
        r = d.compute_poynting_flux({"phasor": r32.det[n]["phasor"]}, cfg.grid.spacing)
        assert rel_l2(g, r) <= TOL


def _phasor_loss(out) -> torch.Tensor:
    return (out.detector_states["objective"]["phasor"].to(torch.complex128).abs() ** 2).sum()


def test_inverse_design_full_size_gradient_vs_finite_differences():
    """The 200 x 200 x 100, 3000-step inverse-design gradient (reversible_fdtd) against central
    finite differences of the float32 GPU forward.

    A one-voxel perturbation of h = 1e-3 moves the objective by about 1e-8 of itself, below
    the float32 rounding of a 3000-step run (the record gives the measured floor: the spread
    between h = 1e-3 and h = 2e-3), so the 16 seeded voxels are checked at h = 0.1 and
    h = 1e-3 is applied along a seeded direction over the whole design region (129,600
    voxels), where the objective moves by about 1e-5 of itself."""
    objects, arrays, params, cfg, _ = scenes.inverse_design(device="cuda")
    p0 = params["design"].detach().clone()
    pg = p0.clone().requires_grad_(True)
    a2, _, _ = fx.apply_params(arrays, objects, {"design": pg})
    _, out = fx.reversible_fdtd(a2, objects, cfg)
    loss = _phasor_loss(out)
    loss.backward()
    grad = pg.grad.detach().double()
    L0 = float(loss.detach())
    fwd_cfg = fx.SimulationConfig(time=cfg.time, grid=cfg.grid, courant_factor=cfg.courant_factor)

    def f(p):
        a, _, _ = fx.apply_params(arrays, objects, {"design": p})
        with torch.no_grad():
            _, o = fx.run_fdtd(a, objects, fwd_cfg)
        return float(_phasor_loss(o))

    assert abs(f(p0) - L0) <= 1e-5 * abs(L0)  # the recording forward and the plain forward agree
    rng = np.random.default_rng(3)
    flat = rng.choice(p0.numel(), size=16, replace=False)
    fds = {}
    for h in (1e-3, 2e-3, 0.1):
        vals = []
        for q in flat.tolist():
            pp, pm = p0.clone(), p0.clone()
            pp.view(-1)[q] += h
            pm.view(-1)[q] -= h
            vals.append((f(pp) - f(pm)) / (2 * h))
        fds[h] = torch.tensor(vals, dtype=torch.float64)
    ad = grad.view(-1)[torch.as_tensor(flat)].cpu()
    v = torch.as_tensor(rng.uniform(-1.0, 1.0, size=tuple(p0.shape)), dtype=torch.float32, device=p0.device)
    h = 1e-3
    fd_dir = (f(p0 + h * v) - f(p0 - h * v)) / (2 * h)
    ad_dir = float((grad * v.double()).sum())
    rec = {
        "loss": L0,
        "voxel_rel_l2_h1e-3": rel_l2(ad, fds[1e-3]),
        "voxel_rel_l2_h0.1": rel_l2(ad, fds[0.1]),
        "noise_floor_rel_l2_h1e-3_vs_2e-3": rel_l2(fds[1e-3], fds[2e-3]),
        "direction_rel_err_h1e-3": abs(ad_dir - fd_dir) / abs(fd_dir),
        "adjoint": ad.tolist(), "fd_h0.1": fds[0.1].tolist(), "fd_h1e-3": fds[1e-3].tolist(),
        "direction": [ad_dir, fd_dir],
    }
    log_result("inverse_design_200x200x100_fd", **rec)
    assert rec["direction_rel_err_h1e-3"] <= 5e-3, rec
    assert rec["voxel_rel_l2_h0.1"] <= 2e-2, rec


def test_inverse_design_scaled_gradient_vs_oracle():
    """A 64 x 64 x 40 copy of the inverse-design scene (design 36 x 36 x 4, 800 steps): the
    parameter gradient against the oracle's restatement of the reference's custom VJP."""
    objects, arrays, params, cfg, _ = scenes.inverse_design(shape=(64, 64, 40), steps=800, design=(36, 36, 4),
                                                            plane=(12, 12), pml=8, device="cpu")
    from tests.test_gpu_adjoint import _to_cuda

    ga = _to_cuda(objects, arrays)
    ie = ga.inv_permittivities.clone().requires_grad_(True)
    _, out = fx.reversible_fdtd(ga.aset("inv_permittivities", ie), objects, cfg)
    (out.detector_states["objective"]["phasor"].abs() ** 2).sum().backward()
    torch.cuda.synchronize()
    g = ie.grad.detach().cpu()
    res = {}
    for dt in (torch.float32, torch.float64):
        sc = O.OracleScene(objects, arrays, cfg, dt)
        fin = O.run(sc, cfg.time_steps_total, record_boundaries=True)
        res[dt] = O.reversible_gradient(sc, fin, {"objective": {"phasor": 2 * fin.det["objective"]["phasor"]}})
    e32, e64 = rel_l2(g, res[torch.float32]), rel_l2(g, res[torch.float64])
    log_result("inverse_design_64x64x40_gradient", grad_rel_l2_vs_fp32=e32, grad_rel_l2_vs_fp64=e64,
               fp32_oracle_vs_fp64=rel_l2(res[torch.float32], res[torch.float64]))
    assert torch.linalg.vector_norm(res[torch.float64]).item() > 0
    assert e32 <= GTOL, (e32, e64)


def _bench_strips(n=64, seed=0):
    """The benchmark's seeded strips: (cells, index, shape, width in um)."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        nx, ny = (int(x) for x in rng.integers(64, 257, size=2))
        nz = int(rng.integers(64, 129))
        w = float(rng.uniform(0.30, 0.80))
        out.append((nx * ny * nz, q, (nx, ny, nz), w))
    return out


def test_batch_smallest_bench_strips_vs_oracle():
    """The two smallest of the 64 seeded strips, batched (graph, autotuned) for their 2000 steps."""
    from fdtdx_gb300.batch import SimulationBatch

    picked = sorted(_bench_strips())[:2]
    sims = []
    for _, _, shape, w in picked:
        o, a, _, c, _ = scenes.strip(shape=shape, width_um=w, steps=2000, device="cuda")
        sims.append((a, o, c))
    b = SimulationBatch(sims)
    b.advance(2000, t0=[0] * len(sims), graph=True, autotune=True)
    torch.cuda.synchronize()
    for (a, o, c), got, (_, q, shape, _) in zip(sims, b.arrays, picked):
        (_, r32), (_, r64) = _oracles(o, a, c)
        compare_states(f"bench_strip_{q}_{shape[0]}x{shape[1]}x{shape[2]}_2000", got, r32, r64, TOL)
    b.close()


def _bench_stream(n_jobs=32, seed=0):
    """The benchmark's seeded request stream: (shape, steps, kind, anisotropic) per request."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n_jobs):
        shp = [int(round(math.exp(rng.uniform(math.log(32), math.log(hi))))) for hi in (384, 384, 192)]
        steps = int(rng.integers(500, 10001))
        kind = "gradient" if rng.uniform() < 0.3 else "forward"
        aniso = bool(rng.uniform() < 0.2)
        specs.append((shp, steps, kind, aniso))
    return specs


def test_served_stream_jobs_vs_oracle():
    """Requests 0 and 23 (forward) and 27 (gradient) of the seeded stream, served together; the
    forward job's fields and detector states and the gradient job's d loss / d inv_eps against
    the oracle."""
    from fdtdx_gb300.serving import Server, random_boxes_job

    specs = _bench_stream()
    ids = {0: 0.0, 27: 0.001, 23: 0.002}
    jobs = []
    for q, arr in ids.items():
        shp, steps, kind, aniso = specs[q]
        jobs.append(random_boxes_job(shp, steps, seed=q, kind=kind, anisotropic=aniso, arrival=arr))
    assert [j.kind for j in jobs] == ["forward", "gradient", "forward"]
    server = Server(budget_bytes=160 * 10**9, max_slots=8, target_chunk_s=0.01)
    server.run(jobs, realtime=False)
    fwd, grad_job = jobs[0], jobs[1]
    o, a, c = fwd.build("cpu", False)
    (_, r32), (_, r64) = _oracles(o, a, c)
    compare_states("served_stream_job0_forward", fwd.result, r32, r64, TOL)
    o, a, c = grad_job.build("cpu", True)
    res = {}
    for dt in (torch.float32, torch.float64):
        sc = O.OracleScene(o, a, c, dt)
        fin = O.run(sc, c.time_steps_total, record_boundaries=True)
        res[dt] = O.reversible_gradient(sc, fin, {"objective": {"phasor": 2 * fin.det["objective"]["phasor"]}})
    g = grad_job.grad.detach().cpu()
    e32, e64 = rel_l2(g, res[torch.float32]), rel_l2(g, res[torch.float64])
    log_result("served_stream_job27_gradient", grad_rel_l2_vs_fp32=e32, grad_rel_l2_vs_fp64=e64)
    assert torch.linalg.vector_norm(res[torch.float64]).item() > 0
    assert e32 <= GTOL, (e32, e64)
