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


def algorithmic_bytes(scene) -> dict:
    """Compulsory float32 bytes per launch of each kernel class (see the design notes)."""
    d = scene.desc
    N = d.nx * d.ny * d.nz
    slab = sum((N // (d.nx, d.ny, d.nz)[d.slabs[s].axis]) * d.slabs[s].thickness for s in range(d.n_slabs))
    e = N * (24 + 12 + 4 * d.n_eps + 4 * d.n_sigma_E) + slab * 16
    h = N * (24 + 12 + 4 * d.n_mu + 4 * d.n_sigma_H) + slab * 16
    det = 0
    for q in range(d.n_detectors):
        dd = d.detectors[q]
        R = (dd.hi[0] - dd.lo[0]) * (dd.hi[1] - dd.lo[1]) * (dd.hi[2] - dd.lo[2])
        C_ = bin(dd.comp_mask).count("1")
        det += R * (4 * C_ + 16 * C_ * max(1, dd.n_freq))
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
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    value = ncell * K * ws / (ms / 1e3)

    # per-kernel device times (CUDA events around each launch group, same stream, same workload)
    prof = (C.c_float * 6)()
    lib = NATIVE.load()
    b = scene.buffers(arrays)
    rc = lib.fdtd_profile_forward(scene.plan, C.byref(b), W + K, 5, prof, C.c_void_p(stream.cuda_stream))
    NATIVE.check(rc, scene.plan, "fdtd_profile_forward")
    groups = ["E update", "E sources", "H update", "H sources", "detectors", "interfaces"]
    times = dict(zip(groups, [float(x) for x in prof]))
    alg = algorithmic_bytes(scene)
    dom = max(("E update", "H update", "detectors"), key=lambda k: times[k])
    peak, peak_kind = _peaks()
    achieved = alg[dom] / (times[dom] / 1e3) / 1e9
    traffic_file = ROOT / "profiles" / "traffic.json"
    traffic = None
    if traffic_file.exists():
        traffic = json.loads(traffic_file.read_text()).get(dom)

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
               "d2h_bytes_per_step": d2h / K, "api": "fdtdx_gb300.run_fdtd"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(budget_s=args.cpu_budget)
    launches = scene.launches_per_step() * K + 1
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
            "workload": f"coupler {shape[0]}x{shape[1]}x{shape[2]} @20nm, 10-cell CPML, CW Gaussian TFSF source, full-volume Ex/Ey/Ez "
                        "phasor + 2 phasor-flux planes (8000-step run; K consecutive steps timed)",
            "cells": ncell,
            "l2": "inputs larger than L2 (fields 384 MB, phasor 768 MB)",
            "parallelism": f"replicas x{ws}",
            "chunk": int(NATIVE.load().fdtd_plan_chunk(scene.plan)),
            "vec": int(NATIVE.load().fdtd_plan_vec(scene.plan)),
            "tma": scene.uses_tma,
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
        },
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


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
        "config": {"workload": "coupler 400x400x200 @20nm (x-slab sample on the host CPU)", "cells": nx * SHAPE[1] * SHAPE[2]},
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
    ap.add_argument("--tma", default="auto", choices=["auto", "0", "1"], help="TMA-pipelined update kernels")
    ap.add_argument("--tz", type=int, default=0)
    ap.add_argument("--ty", type=int, default=0)
    ap.add_argument("--stages", type=int, default=0)
    ap.add_argument("--tchunk", type=int, default=0)
    ap.add_argument("--boundary", default="pml", help="boundary type of the workload (profiling ablations)")
    ap.add_argument("--no-phasor", action="store_true", help="drop the full-volume phasor (profiling ablations)")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
