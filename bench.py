"""Benchmark: cell-updates/s of the FDTD time step on the two-strip coupler workload.

Workload (one "step" = one Yee time step of the whole hot path): 400 x 400 x 200 cells at
20 nm, 10-cell CPML on all faces, SiO2 with two Si strips, a CW Gaussian TFSF plane source,
a full-volume phasor detector of Ex/Ey/Ez and two phasor-flux planes (8000-step run; the
timed steps are K consecutive steps of it).  Inputs (fields 384 MB each, the 768 MB phasor)
are larger than the 129 MB L2, so no flush is needed between steps.

Arms:
  default            the GB300 library (CUDA-graph replayed steps), inputs resident in HBM
                     for ``value``; ``e2e`` goes through ``run_fdtd`` with the permittivity
                     uploaded from pinned host memory and the flux-plane phasors read back.
  --impl reference   the CPU restatement of the reference (oracle/fdtd_oracle.py, torch-CPU
                     float32, all host threads) on a bounded x-slab sample of the same scene.

Multi-GPU (torchrun): replicas only -- each rank runs the same simulation on its own GPU,
no data exchange (the configs are single-GPU; ``scaling: weak``).
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import torch

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s"
SHAPE = (400, 400, 200)
T_TOTAL = 8000


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(ms: float, dev) -> float:
    """The slowest rank's timed-region length: the job's steps are done when the last rank's are."""
    import torch.distributed as dist

    t = torch.tensor([ms], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _job_rate(ncell: int, steps: int, ws: int, ms: float) -> float:
    """Whole-job cell-updates/s: every rank advances its own replica of ``ncell`` cells by
    ``steps`` steps within the slowest rank's ``ms``."""
    return ncell * steps * ws / (ms / 1e3)


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms",
                 "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def workload_name(shape=SHAPE) -> str:
    """The workload string both arms print (the reference arm times a bounded x-slab sample of
    this same scene; its ``cpu_baseline.sample`` says which)."""
    return (f"coupler {shape[0]}x{shape[1]}x{shape[2]} @20nm, 10-cell CPML, CW Gaussian TFSF source, full-volume "
            "Ex/Ey/Ez phasor + 2 phasor-flux planes (8000-step run; K consecutive steps timed)")


def _fused(dd) -> bool:
    """E-only phasor / field detectors without volume reduction ride in the H half-step."""
    return dd.kind in (1, 0) and (dd.comp_mask & 56) == 0 and not dd.reduce_volume


def algorithmic_bytes(scene) -> dict:
    """Compulsory float32 bytes per launch group: E update (E r/w, H, inv_eps, sigma, psi_E
    r/w on slab cells), H update (H r/w, E, inv_mu, sigma, psi_H r/w, plus the read-modify-
    write of the detectors fused into it), detectors (the other detectors' samples)."""
    import fdtdx_gb300._native as NATIVE

    d = scene.desc
    N = d.nx * d.ny * d.nz
    slab = sum((N // (d.nx, d.ny, d.nz)[d.slabs[s].axis]) * d.slabs[s].thickness for s in range(d.n_slabs))
    e = N * (24 + 12 + 4 * d.n_eps + 4 * d.n_sigma_E) + slab * 16
    h = N * (24 + 12 + 4 * d.n_mu + 4 * d.n_sigma_H) + slab * 16
    det = 0
    n_fused = 0
    for q in range(d.n_detectors):
        dd = d.detectors[q]
        R = (dd.hi[0] - dd.lo[0]) * (dd.hi[1] - dd.lo[1]) * (dd.hi[2] - dd.lo[2])
        C_ = bin(dd.comp_mask).count("1")
        if dd.kind == NATIVE.DET_PHASOR:
            b = R * 16 * C_ * max(1, dd.n_freq)  # complex64 read + write per component and frequency
        else:
            b = R * 4 * C_
        if _fused(dd) and n_fused < 2:
            h += b
            n_fused += 1
        else:
            det += b + R * 4 * C_  # samples gathered from the fields
    return {"E update": e, "H update": h, "detectors": det}


def run_gpu(args):
    import torch.distributed as dist

    import fdtdx_gb300 as fx
    from fdtdx_gb300 import _native as NATIVE, scenes
    from fdtdx_gb300.fdtd import get_scene

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    shape = tuple(int(x) for x in args.shape.split(",")) if args.shape else SHAPE
    objects, arrays, _, cfg, _ = scenes.coupler(shape=shape, steps=T_TOTAL, device=dev, boundary=args.boundary,
                                                full_phasor=not args.no_phasor)
    arrays = arrays.reset()
    scene = get_scene(objects, arrays, cfg)
    if args.tma == "0":
        scene.tune_tma(False)
    elif args.tma == "1" or args.tz or args.ty or args.stages or args.tchunk:
        scene.tune_tma(True, args.tz, args.ty, args.stages, args.tchunk)
    if args.chunk or args.vec:
        scene.tune(args.chunk, args.vec)
    if args.shell_chunk or args.shell_vec:
        scene.tune_shell(args.shell_chunk, args.shell_vec)
    if args.shell_tma >= 0:
        scene.tune_shell_tma(args.shell_tma, args.pml_tz, args.pml_chunk)
    ncell = shape[0] * shape[1] * shape[2]
    W, K = args.warmup, args.steps
    if W + K + 8 > T_TOTAL:
        raise SystemExit("warmup + steps must stay below the 8000-step run")
    stream = torch.cuda.current_stream()
    scene.forward(arrays, 0, W)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        scene.forward(arrays, W, K)
        ev1.record(stream)
        torch.cuda.synchronize()
    scene.status()
    ms = ev0.elapsed_time(ev1)
    if ws > 1:
        ms = _max_over_ranks(ms, dev)
        dist.barrier()
    value = _job_rate(ncell, K, ws, ms)

    # per-kernel device times (CUDA events around each launch group, same stream, same workload)
    prof = (C.c_float * 8)()
    lib = NATIVE.load()
    b = scene.buffers(arrays)
    rc = lib.fdtd_profile_forward(scene.plan, C.byref(b), W + K, 5, prof, C.c_void_p(stream.cuda_stream))
    NATIVE.check(rc, scene.plan, "fdtd_profile_forward")
    parts = ["E core", "E shell", "E sources", "H core", "H shell", "H sources", "detectors", "interfaces"]
    split = dict(zip(parts, [float(x) for x in prof]))
    times = {"E update": split["E core"] + split["E shell"], "E sources": split["E sources"],
             "H update": split["H core"] + split["H shell"], "H sources": split["H sources"],
             "detectors": split["detectors"], "interfaces": split["interfaces"]}
    alg = algorithmic_bytes(scene)
    dom = max(("E update", "H update", "detectors"), key=lambda k: times[k])
    peak, peak_kind = _peaks()
    achieved = alg[dom] / (times[dom] / 1e3) / 1e9
    traffic = None
    traffic_file = ROOT / "profiles" / "coupler_traffic.txt"
    if traffic_file.exists() and shape == SHAPE:
        for ln in traffic_file.read_text().splitlines():
            if ln.startswith(dom + " "):
                traffic = int(ln.split()[-1])

    # end to end through run_fdtd: permittivity from pinned host memory, flux phasors read back
    cfg_e2e = fx.SimulationConfig(time=K * cfg.time_step_duration, grid=cfg.grid, courant_factor=cfg.courant_factor)
    host_eps = arrays.inv_permittivities.detach().to("cpu").pin_memory()
    base = arrays

    def e2e_once():
        ie = host_eps.to(dev, non_blocking=True)
        arr = base.aset("inv_permittivities", ie)
        _, out = fx.run_fdtd(arr, objects, cfg_e2e)
        res = [out.detector_states[n]["phasor"].to("cpu") for n in ("flux1", "flux2")]  # the flux planes' phasors
        return res

    e2e = None
    if not args.no_e2e:
        e2e_once()
        torch.cuda.synchronize()
        reps = 2
        t0 = time.perf_counter()
        for _ in range(reps):
            res = e2e_once()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / reps
        h2d = host_eps.numel() * 4
        d2h = sum(r.numel() * 8 for r in res)
        e2e = {"value": ncell * K * ws / e2e_s, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d / K,
               "d2h_bytes_per_step": d2h / K, "api": "fdtdx_gb300.run_fdtd",
               "copies": "in: inv_permittivities from pinned host memory each call; out: the two flux-plane "
                         "phasors (the run's result); E, H and the full-volume phasor stay on the device"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(budget_s=args.cpu_budget)
    launches = scene.launches_per_step() * K + 1
    # the gradient, batch and serving measurements, each on its own workload (reported, not the headline)
    extra = {}
    scene.close()
    del arrays, base, host_eps
    torch.cuda.empty_cache()
    if ws > 1:  # the secondary measurements are single-GPU workloads: the headline alone scales
        args.no_gradient = args.no_batch = args.no_serving = True
    if not args.no_gradient:
        extra["gradient"] = bench_gradient(dev)
        torch.cuda.empty_cache()
    if not args.no_batch:
        extra["batch"] = bench_batch(dev, args.batch_sims, args.batch_steps)
        torch.cuda.empty_cache()
    if not args.no_serving:
        cap = extra["batch"]["batched_cell_updates_per_s"] if "batch" in extra else value
        extra["serving"] = bench_serving(cap, args.serve_jobs)
        torch.cuda.empty_cache()
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "cell-updates/s",
        "n_gpus": ws,
        "steps": K,
        "warmup": W,
        "ms_per_step": ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene builder)",
        "config": {
            "workload": workload_name(shape),
            "cells": ncell,
            "l2": "inputs larger than L2 (fields 384 MB, phasor 768 MB)",
            "parallelism": f"replicas x{ws}",
            "chunk": int(NATIVE.load().fdtd_plan_chunk(scene.plan)),
            "vec": int(NATIVE.load().fdtd_plan_vec(scene.plan)),
            "tma": scene.uses_tma,
            "shell_tma": scene.shell_tma,
            "hbm_gbs_effective": round(sum(alg.values()) / (ms / K / 1e3) / 1e9, 1),
        },
        "roofline": {
            "kernel": dom,
            "bound": "hbm",
            "achieved": round(achieved, 1),
            "peak": peak,
            "peak_kind": peak_kind,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "traffic": traffic,
            "alg_bytes_per_launch": alg[dom],
            "kernel_ms": {k: round(v, 4) for k, v in times.items()},
            "launch_ms": {k: round(v, 4) for k, v in split.items()},
        },
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    line.update(extra)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


def bench_gradient(dev, steps: int = 3000) -> dict:
    """Inverse-design gradient: 200x200x100 @25 nm, 10-cell CPML, 3000 steps, 120x120x9 design
    region, pulsed plane source, sum |phasor|^2 over a 40x40 plane; d loss / d params through
    reversible_fdtd (forward with interface recording, then the T+1-step adjoint)."""
    import fdtdx_gb300 as fx
    from fdtdx_gb300 import scenes
    from fdtdx_gb300.fdtd import _materials_detached, get_scene

    objects, arrays, params, cfg, _ = scenes.inverse_design(steps=steps, device=dev)
    T = cfg.time_steps_total
    N = 200 * 200 * 100

    def once():
        p = params["design"].detach().clone().requires_grad_(True)
        a2, _, _ = fx.apply_params(arrays, objects, {"design": p})
        _, out = fx.reversible_fdtd(a2, objects, cfg)
        loss = (out.detector_states["objective"]["phasor"].abs() ** 2).sum()
        loss.backward()
        return p.grad

    once()  # plans built, graphs captured
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = once()
    torch.cuda.synchronize()
    total = time.perf_counter() - t0
    # split: forward with recording alone, on the cached scene
    work = _materials_detached(fx.apply_params(arrays, objects, params)[0]).reset()
    scene = get_scene(objects, work, cfg, record_interfaces=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    scene.forward(work, 0, T)
    e1.record()
    torch.cuda.synchronize()
    fwd = e0.elapsed_time(e1) / 1e3
    return {
        "workload": f"inverse design 200x200x100 @25nm, 10-cell CPML, {T} steps, 120x120x9 design, plane pulse, "
                    "|phasor|^2 on a 40x40 plane; gradient via reversible_fdtd (T+1 adjoint steps)",
        "gradient_s": round(total, 4),
        "forward_s": round(fwd, 4),
        "adjoint_s": round(total - fwd, 4),
        "forward_cell_updates_per_s": N * T / fwd,
        "adjoint_cell_updates_per_s": N * (T + 1) / max(1e-9, total - fwd),
        "grad_finite": bool(torch.isfinite(g).all().item()),
        }


def _strip_sims(n: int, steps: int, dev, seed: int = 0, lo=(64, 64, 64), hi=(256, 256, 128), pml: int = 10):
    """Seeded strips (uniform integer sizes per axis in [lo, hi], width uniform in 0.30-0.80 um)."""
    import numpy as np

    from fdtdx_gb300 import scenes

    rng = np.random.default_rng(seed)
    sims, cells = [], 0
    for _ in range(n):
        nx, ny = (int(x) for x in rng.integers((lo[0], lo[1]), (hi[0] + 1, hi[1] + 1)))
        nz = int(rng.integers(lo[2], hi[2] + 1))
        w = float(rng.uniform(0.30, 0.80))
        o, a, _, c, _ = scenes.strip(shape=(nx, ny, nz), width_um=w, steps=steps, device=dev, pml=pml)
        sims.append((a, o, c))
        cells += nx * ny * nz
    return sims, cells


def _zero_state(arrays) -> None:
    """Fields, psi and detector states back to zero in place (a fresh run on the same buffers,
    so captured CUDA graphs stay valid)."""
    f = arrays.fields
    f.E.zero_()
    f.H.zero_()
    for n in f.psi_E:
        for t in (*f.psi_E[n], *f.psi_H[n]):
            t.zero_()
    for st in arrays.detector_states.values():
        for v in st.values():
            v.zero_()


def _batch_case(sims, cells, steps: int) -> dict:
    """One batch of ``sims`` against the same runs one at a time, plans, batch tables, tile
    tuning and CUDA-graph capture all done before either timer starts."""
    from fdtdx_gb300.batch import SimulationBatch
    from fdtdx_gb300.engine import Scene
    from fdtdx_gb300.fdtd import _materials_detached

    work = cells * steps
    # one at a time: every plan built and its graph captured first, then the runs back to back
    seq = []
    for a, o, c in sims:
        w = _materials_detached(a).reset()
        sc = Scene(o, w, c)
        sc.forward(w, 0, 64)
        _zero_state(w)
        seq.append((sc, w))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for sc, w in seq:
        sc.forward(w, 0, steps)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    for sc, _ in seq:
        sc.close()
    del seq
    torch.cuda.empty_cache()
    # batched: tiles tuned on real steps and the graph captured, then the state zeroed
    b = SimulationBatch(sims)
    b.advance(min(400, steps), t0=[0] * len(sims), graph=True, autotune=True)
    b.advance(64, graph=True, autotune=False)
    for w in b.arrays:
        _zero_state(w)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.advance(steps, t0=[0] * len(sims), graph=True, autotune=False)
    torch.cuda.synchronize()
    bt = time.perf_counter() - t0
    tune = b.tuning()
    launches = b.launches_per_step()
    # each execution mode on its own (CUDA graph where the mode has one), fewer steps
    mode_steps = min(steps, 400)
    modes = {}
    for mode in ("persistent", "branches", "fused"):
        b.set_mode(mode)
        b.advance(64, t0=[0] * len(sims), graph=True, autotune=False)
        for w in b.arrays:
            _zero_state(w)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.advance(mode_steps, t0=[0] * len(sims), graph=True, autotune=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        # launches per batch step; the fused mode reports 1: one launch runs all the steps of a call
        modes[mode] = {"steps": mode_steps, "s": round(dt, 4), "cell_updates_per_s": cells * mode_steps / dt,
                       "launches_per_step": b.launches_per_step()}
    b.close()
    return {
        "cells_total": cells,
        "batched_cell_updates_per_s": work / bt,
        "sequential_cell_updates_per_s": work / seq_s,
        "speedup_vs_sequential": seq_s / bt,
        "batched_s": round(bt, 3),
        "sequential_s": round(seq_s, 3),
        "launches_per_batch_step": launches,
        "tiles": tune,
        "modes": modes,
    }


def _strip_bytes_per_step(sims) -> float:
    """Algorithmic bytes of one step of every simulation (the per-launch-group formula summed)."""
    from fdtdx_gb300.engine import Scene

    tot = 0
    for a, o, c in sims:
        sc = Scene(o, a, c)
        tot += sum(algorithmic_bytes(sc).values())
    return float(tot)


def bench_batch(dev, n_sims: int = 64, steps: int = 2000) -> dict:
    """64 Si strips of seeded uneven grids (64..256 x 64..256 x 64..128 @25 nm, 10-cell CPML,
    2000 steps, pulsed Gaussian source, transmitted phasor flux): one batch (CUDA graph,
    autotuned tiles) against the same runs one at a time; and the same for 64 small strips
    (32..96 per axis, 8-cell CPML), where a run alone is bound by launches, not bandwidth.
    Setup (plans, batch tables, tuning, graph capture) is outside both timers."""
    peak, _ = _peaks()
    sims, cells = _strip_sims(n_sims, steps, dev)
    out = {"workload": f"{n_sims} Si strips, seeded grids 64-256 x 64-256 x 64-128 @25nm, 10-cell CPML, {steps} steps, "
                       "pulsed Gaussian source, transmitted phasor flux"}
    bps = _strip_bytes_per_step(sims)
    r = _batch_case(sims, cells, steps)
    r["batched_roofline_frac"] = round(bps * steps / r["batched_s"] / 1e9 / peak, 4)
    out.update(r)
    del sims
    torch.cuda.empty_cache()
    small, scells = _strip_sims(n_sims, steps, dev, seed=1, lo=(32, 32, 32), hi=(96, 96, 96), pml=8)
    sb = _strip_bytes_per_step(small)
    rs = _batch_case(small, scells, steps)
    rs["batched_roofline_frac"] = round(sb * steps / rs["batched_s"] / 1e9 / peak, 4)
    rs["sequential_roofline_frac"] = round(sb * steps / rs["sequential_s"] / 1e9 / peak, 4)
    rs["workload"] = f"{n_sims} small Si strips, seeded grids 32-96 per axis @25nm, 8-cell CPML, {steps} steps"
    out["small_grids"] = rs
    return out


def bench_batch_modes(dev, n_sims: int = 32, steps: int = 6) -> dict:
    """Profiling case of the batch execution modes on small strips (32..96 per axis, 8-cell
    CPML), direct launches: per mode a 2-step warm-up call, then one timed call of ``steps``
    steps.  The fused mode runs first, so its timed call is the second k_batch_fused launch and
    the persistent mode's k_batch_update launches follow it."""
    from fdtdx_gb300.batch import SimulationBatch

    sims, cells = _strip_sims(n_sims, steps + 2, dev, seed=1, lo=(32, 32, 32), hi=(96, 96, 96), pml=8)
    b = SimulationBatch(sims)
    out = {"workload": f"{n_sims} small Si strips, seeded grids 32-96 per axis @25nm, 8-cell CPML", "cells": cells}
    for mode in ("fused", "persistent", "branches"):
        b.set_mode(mode)
        b.advance(2, t0=[0] * n_sims, graph=False, autotune=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.advance(steps, graph=False, autotune=False)
        torch.cuda.synchronize()
        out[mode] = {"steps": steps, "ms": round((time.perf_counter() - t0) * 1e3, 3)}
    b.close()
    return out


def bench_serving(capacity: float, n_jobs: int = 200, seed: int = 0, load: float = 1.5) -> dict:
    """Poisson stream: grids log-uniform in [32,384]x[32,384]x[32,192] @50 nm, steps uniform
    in [500, 10000], 70% forward / 30% forward+gradient, random boxes (20% diagonal-
    anisotropic, per-axis eps in [2, 12]), 160 GB admission budget.  The offered load is
    ``load`` x the measured batched capacity, so both arms run saturated and their aggregate
    throughputs and latencies compare; served (continuous batching) against one at a time."""
    import numpy as np

    from fdtdx_gb300.serving import Server, estimate_footprint, latency_stats, random_boxes_job, run_one_at_a_time

    budget = 160 * 10**9

    def make():
        rng = np.random.default_rng(seed)
        specs = []
        for _ in range(n_jobs):
            shp = [int(round(math.exp(rng.uniform(math.log(32), math.log(hi))))) for hi in (384, 384, 192)]
            steps = int(rng.integers(500, 10001))
            kind = "gradient" if rng.uniform() < 0.3 else "forward"
            aniso = bool(rng.uniform() < 0.2)
            specs.append((shp, steps, kind, aniso))
        return [random_boxes_job(shp, steps, seed=seed * 1000 + q, kind=kind, anisotropic=aniso)
                for q, (shp, steps, kind, aniso) in enumerate(specs)]

    jobs = make()
    keep = [j for j in jobs if estimate_footprint(j) <= budget]
    work = sum(j.cells * j.steps * (4.5 if j.kind == "gradient" else 1.0) for j in keep)
    rate = load * capacity / (work / len(keep))  # jobs per second
    rng = np.random.default_rng(seed + 1)
    t = 0.0
    arrivals = []
    for _ in keep:
        t += float(rng.exponential(1.0 / rate))
        arrivals.append(t)
    for j, a in zip(keep, arrivals):
        j.arrival = a
    # at most eight jobs in flight: a saturated stream keeps its tail close to first-come order
    # (measured on this stream: p99 38.8 s at 8 slots, 44.4 s at 16, 53.5 s at 64)
    server = Server(budget_bytes=budget, max_slots=8, target_chunk_s=0.05, keep_results=False)
    server.run(keep, realtime=True)
    served = latency_stats(keep)
    served_work = server.forward_cell_updates + server.adjoint_cell_updates
    torch.cuda.empty_cache()
    # the same stream one at a time
    keep2 = [j for j in make() if estimate_footprint(j) <= budget]
    for j, a in zip(keep2, arrivals):
        j.arrival = a
    t0 = time.perf_counter()
    run_one_at_a_time(keep2, realtime=True, keep_results=False)
    plain_s = time.perf_counter() - t0
    plain = latency_stats(keep2)
    return {
        "workload": f"{len(keep)} jobs (of {n_jobs}; larger than the budget dropped), grids log-uniform 32-384 x 32-384 "
                    "x 32-192 @50nm, steps 500-10000, 70% forward / 30% gradient, 20% diagonal-anisotropic, "
                    f"160 GB budget, Poisson arrivals at {load}x the batched capacity",
        "rate_jobs_per_s": rate,
        "served": {"p50_s": served["p50_s"], "p99_s": served["p99_s"], "mean_s": served["mean_s"],
                   "makespan_s": server.makespan, "cell_updates_per_s": served_work / server.makespan},
        "one_at_a_time": {"p50_s": plain["p50_s"], "p99_s": plain["p99_s"], "mean_s": plain["mean_s"],
                          "makespan_s": plain_s, "cell_updates_per_s": served_work / plain_s},
        "gradient_jobs": sum(1 for j in keep if j.kind == "gradient"),
    }


def _oracle_rate(nx: int, steps: int, warmup: int = 1):
    """cell-updates/s of the CPU restatement on an x-slab of the coupler scene."""
    from fdtdx_gb300 import scenes
    from oracle import fdtd_oracle as O

    objects, arrays, _, cfg, _ = scenes.coupler(shape=(nx, SHAPE[1], SHAPE[2]), steps=T_TOTAL, device="cpu")
    sc = O.OracleScene(objects, arrays, cfg, torch.float32)
    st = sc.init_state()
    with torch.no_grad():
        for _ in range(warmup):
            st = O.forward(sc, st)
        t0 = time.perf_counter()
        for _ in range(steps):
            st = O.forward(sc, st)
        dt = time.perf_counter() - t0
    return nx * SHAPE[1] * SHAPE[2] * steps / dt, dt


def cpu_baseline(budget_s: float = 20.0) -> dict:
    torch.set_num_threads(os.cpu_count() or 1)
    nx = 60
    rate, _ = _oracle_rate(nx, 1, warmup=1)
    steps = max(1, int(budget_s * rate / (nx * SHAPE[1] * SHAPE[2])))
    steps = min(steps, 50)
    rate, dt = _oracle_rate(nx, steps, warmup=0)
    return {"value": rate, "unit": "cell-updates/s", "cores": torch.get_num_threads(), "kind": "port",
            "sample": f"oracle float32, {steps} steps of a {nx}x{SHAPE[1]}x{SHAPE[2]} x-slab of the coupler scene "
                      f"({dt:.1f} s)"}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    torch.set_num_threads(os.cpu_count() or 1)
    W, K = args.warmup, args.steps
    # size the x-slab so the whole run stays near args.cpu_budget seconds
    probe, _ = _oracle_rate(32, 1, warmup=1)
    per_step_budget = max(0.5, args.ref_budget / max(1, W + K))
    nx = int(max(32, min(SHAPE[0], per_step_budget * probe / (SHAPE[1] * SHAPE[2]))))
    from fdtdx_gb300 import scenes
    from oracle import fdtd_oracle as O

    objects, arrays, _, cfg, _ = scenes.coupler(shape=(nx, SHAPE[1], SHAPE[2]), steps=T_TOTAL, device="cpu")
    sc = O.OracleScene(objects, arrays, cfg, torch.float32)
    st = sc.init_state()
    with torch.no_grad():
        for _ in range(W):
            st = O.forward(sc, st)
        t0 = time.perf_counter()
        for _ in range(K):
            st = O.forward(sc, st)
        dt = time.perf_counter() - t0
    val = nx * SHAPE[1] * SHAPE[2] * K / dt
    sample = f"oracle float32 on a {nx}x{SHAPE[1]}x{SHAPE[2]} x-slab of the coupler scene, {K} steps"
    line = {
        "metric": METRIC, "value": val, "unit": "cell-updates/s", "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": dt / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene builder)", "impl": "reference",
        "config": {"workload": workload_name(), "cells": SHAPE[0] * SHAPE[1] * SHAPE[2],
                   "sample_cells": nx * SHAPE[1] * SHAPE[2]},
        "cpu_baseline": {"value": val, "unit": "cell-updates/s", "cores": torch.get_num_threads(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": val, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--ref-budget", type=float, default=120.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--shape", default="", help="grid override nx,ny,nz (profiling cases)")
    ap.add_argument("--chunk", type=int, default=0, help="x planes per update block (0: plan default)")
    ap.add_argument("--vec", type=int, default=0, help="z cells per thread (0: plan default)")
    ap.add_argument("--shell-chunk", type=int, default=0, help="x planes per CPML shell block (0: plan default)")
    ap.add_argument("--shell-vec", type=int, default=0, help="z cells per CPML shell thread (0: plan default)")
    ap.add_argument("--tma", default="auto", choices=["auto", "0", "1"], help="TMA-pipelined update kernels")
    ap.add_argument("--shell-tma", type=int, default=-1, choices=[-1, 0, 1, 2, 3, 4, 5],
                    help="CPML slab cells on the TMA kernels: 0 none, 1 x and y slabs, 2 all, 3 split "
                         "(plain TMA over the grid + per-axis corrections), 4 split with the z slabs in the "
                         "tiles, 5 mode 4 for E and 3 for H (-1: default)")
    ap.add_argument("--pml-tz", type=int, default=0, help="z extent of the whole-grid TMA tile (shell mode 2)")
    ap.add_argument("--pml-chunk", type=int, default=0, help="x planes per block of the slab-cell TMA launch")
    ap.add_argument("--tz", type=int, default=0)
    ap.add_argument("--ty", type=int, default=0)
    ap.add_argument("--stages", type=int, default=0)
    ap.add_argument("--tchunk", type=int, default=0)
    ap.add_argument("--boundary", default="pml", help="boundary type of the workload (profiling ablations)")
    ap.add_argument("--no-phasor", action="store_true", help="drop the full-volume phasor (profiling ablations)")
    ap.add_argument("--no-gradient", action="store_true", help="skip the inverse-design gradient measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-simulation batch measurement")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-stream measurement")
    ap.add_argument("--batch-sims", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=2000)
    ap.add_argument("--serve-jobs", type=int, default=200)
    ap.add_argument("--case", default="all", choices=["all", "gradient", "batch", "batch-modes", "serving"],
                    help="run one secondary measurement alone and print its record (profiling)")
    ap.add_argument("--grad-steps", type=int, default=3000, help="steps of the gradient case (profiling: fewer)")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.case != "all":
        torch.cuda.set_device(0)
        dev = torch.device("cuda", 0)
        if args.case == "gradient":
            out = bench_gradient(dev, args.grad_steps)
        elif args.case == "batch":
            out = bench_batch(dev, args.batch_sims, args.batch_steps)
        elif args.case == "batch-modes":
            out = bench_batch_modes(dev, args.batch_sims, args.batch_steps)
        else:
            out = bench_serving(2.0e10, args.serve_jobs)
        print(json.dumps({"case": args.case, **out}))
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
