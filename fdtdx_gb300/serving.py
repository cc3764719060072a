"""Serving loop: forward and gradient jobs admitted by HBM footprint, continuously batched.

There is no serving layer in fdtdx; this module is the GB300 runtime around the native
path for a stream of independent simulation requests:

* admission by HBM footprint (``fdtd_footprint_bytes``, which counts fields, materials,
  psi, detector states, the interface recording and, for gradient jobs, the adjoint
  buffers) against a budget, plus a slot limit; FIFO with bounded backfill (a job that
  does not fit may be overtaken by later ones at most ``max_bypass`` times);
* every admitted job keeps its state on the device until it completes;
* continuous batching: all jobs in their forward phase advance together through one
  ``fdtd_batch_forward`` call per chunk (the batch is rebuilt whenever a job joins or
  leaves), while gradient jobs in their adjoint phase run ``fdtd_adjoint`` chunks on
  adjoint lanes (streams of their own), so the kinds of work overlap on the GPU; every lane
  gets its next chunk when its CUDA event says the last one finished, with no device-wide
  wait, and admitted jobs are placed by a worker thread on a side stream meanwhile;
* cancellation of queued and running jobs, host snapshots of a running job's state, and
  per-job divergence detection (a non-finite job fails alone);
* per-job latency (arrival to completion) and aggregate throughput are recorded.

The scheduling logic (``Scheduler``) is host-only and unit-tested without a GPU.
"""

from __future__ import annotations

import collections
import math
import time
from dataclasses import dataclass
from typing import Callable

import torch

from fdtdx_gb300.config import SimulationConfig
from fdtdx_gb300.container import ArrayContainer, ObjectContainer


def phasor_power_loss(name: str) -> Callable[[dict], torch.Tensor]:
    """Objective sum |phasor|^2 of detector ``name`` (the inverse-design form)."""

    def loss(det: dict) -> torch.Tensor:
        return (det[name]["phasor"].abs() ** 2).sum()

    return loss


# build(device, with_recorder) -> (objects, arrays, config): places the job's simulation on
# `device`; gradient jobs are built with an interface recorder on the GPU.
Builder = Callable[[str, bool], tuple[ObjectContainer, ArrayContainer, SimulationConfig]]


@dataclass
class Job:
    """One request: how to place its simulation and what to compute."""

    build: Builder
    kind: str = "forward"                       # "forward" or "gradient"
    loss: Callable[[dict], torch.Tensor] | None = None  # gradient jobs: scalar of the detector states
    arrival: float = 0.0                        # seconds after the stream start
    # filled in by estimate_footprint / the server
    id: int = -1
    footprint: int = 0
    n_cells: int = 0
    steps: int = 0
    objects: ObjectContainer | None = None
    arrays: ArrayContainer | None = None
    config: SimulationConfig | None = None
    detectors: dict | None = None               # gradient jobs: the final detector states
    phase: str = "queued"                       # queued, forward, adjoint, done, cancelled, failed
    t_fwd: int = 0                              # forward steps done
    t_adj: int = 0                              # adjoint steps left
    bypassed: int = 0
    t_admit: float = math.nan
    t_done: float = math.nan
    result: ArrayContainer | None = None
    grad: torch.Tensor | None = None
    loss_value: float | None = None
    scene: object = None
    state: ArrayContainer | None = None
    lam: dict | None = None
    cancel_requested: bool = False
    error: str | None = None                    # why a failed job failed
    inflight: int = 0                           # steps of a chunk issued and not yet accounted

    @property
    def cells(self) -> int:
        return self.n_cells

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def random_boxes_job(shape, steps: int, seed: int, kind: str = "forward", anisotropic: bool = False,
                     arrival: float = 0.0, **kw) -> Job:
    """A serving request over ``scenes.serving_job`` (random boxes, dipole, E phasor plane)."""
    from fdtdx_gb300 import scenes

    def build(device: str, with_recorder: bool):
        o, a, _p, c, _i = scenes.serving_job(shape=tuple(shape), steps=steps, seed=seed, anisotropic=anisotropic,
                                             gradient=kind == "gradient", with_recorder=with_recorder,
                                             device=device, **kw)
        return o, a, c

    loss = phasor_power_loss("objective") if kind == "gradient" else None
    return Job(build=build, kind=kind, loss=loss, arrival=arrival)


def estimate_footprint(job: Job) -> int:
    """The job's device footprint from a host-side build of its description (no device
    memory is touched): ``fdtd_footprint_bytes`` of its plan description."""
    from fdtdx_gb300.engine import Scene

    objects, arrays, config = job.build("cpu", False)
    scene = Scene(objects, arrays, config, record_interfaces=job.kind == "gradient")
    job.footprint = scene.footprint_bytes()
    n = objects.volume.grid_shape
    job.n_cells = n[0] * n[1] * n[2]
    job.steps = config.time_steps_total
    return job.footprint


class Scheduler:
    """Admission and phase bookkeeping of the serving loop (host only)."""

    def __init__(self, budget_bytes: int, max_slots: int = 64, max_bypass: int = 8):
        self.budget = int(budget_bytes)
        self.max_slots = int(max_slots)
        self.max_bypass = int(max_bypass)
        self.queue: collections.deque[Job] = collections.deque()
        self.active: list[Job] = []
        self.used = 0
        self.done: list[Job] = []

    def arrive(self, job: Job) -> None:
        if job.footprint > self.budget:
            raise ValueError(f"job {job.id} needs {job.footprint} bytes, more than the whole budget {self.budget}")
        job.phase = "queued"
        self.queue.append(job)

    def admit(self, now: float) -> list[Job]:
        """Admit queued jobs that fit, in arrival order; a job that does not fit lets later
        ones pass at most ``max_bypass`` times, after which admission waits for it."""
        admitted = []
        blocked = False
        for job in list(self.queue):
            if len(self.active) >= self.max_slots:
                break
            fits = self.used + job.footprint <= self.budget
            if fits and not blocked:
                self.queue.remove(job)
                self.active.append(job)
                self.used += job.footprint
                job.phase = "forward"
                job.t_admit = now
                admitted.append(job)
            elif not fits:
                job.bypassed += 1
                if job.bypassed > self.max_bypass:
                    blocked = True  # reserve: nothing behind it is admitted until it fits
        return admitted

    def forward_jobs(self) -> list[Job]:
        return [j for j in self.active if j.phase == "forward"]

    def adjoint_jobs(self) -> list[Job]:
        return [j for j in self.active if j.phase == "adjoint"]

    def forward_chunk(self, cap: int) -> int:
        """Steps the forward batch can advance: at most ``cap`` and no job past its end."""
        fw = self.forward_jobs()
        if not fw:
            return 0
        return max(1, min(cap, min(j.steps - j.t_fwd for j in fw)))

    def advanced(self, job: Job, n: int) -> None:
        job.t_fwd += n

    def forward_finished(self, job: Job) -> bool:
        return job.t_fwd >= job.steps

    def start_adjoint(self, job: Job) -> None:
        job.phase = "adjoint"
        job.t_adj = job.steps + 1  # the reference's backward loop runs t = T-1 .. -1

    def complete(self, job: Job, now: float, phase: str = "done") -> None:
        """A job leaves the active set ("done", "cancelled" or "failed") and frees its budget."""
        job.phase = phase
        job.t_done = now
        self.active.remove(job)
        self.used -= job.footprint
        self.done.append(job)

    def withdraw(self, job: Job, now: float) -> bool:
        """Removes a queued job (cancellation before admission); False when it is not queued."""
        if job not in self.queue:
            return False
        self.queue.remove(job)
        job.phase = "cancelled"
        job.t_done = now
        self.done.append(job)
        return True

    def idle(self) -> bool:
        return not self.queue and not self.active


class Server:
    """The GPU serving loop over a list of timed jobs (``Job.arrival`` in seconds)."""

    def __init__(self, budget_bytes: int = 160 * 10**9, max_slots: int = 8, target_chunk_s: float = 0.05,
                 autotune: bool = True, adjoint_lanes: int = 4, keep_results: bool = True):
        """``keep_results=False`` returns each finished job's detector states on the host (in
        ``Job.detectors``) and frees its device state, as a service answering many requests does.
        ``max_slots`` bounds the jobs in flight: few enough that a saturated stream is served close
        to first-come order (its tail stays short), enough that small grids still fill the device
        together."""
        self.sched = Scheduler(budget_bytes, max_slots)
        self.keep_results = keep_results
        self.adjoint_lanes = max(1, int(adjoint_lanes))
        self.target = float(target_chunk_s)
        self.autotune = autotune
        self._tile = None
        self._batch = None
        self._members: tuple = ()
        self.rate = 2.0e10  # cell-updates/s estimate, refined online
        self.adj_rate = 6.0e9
        self.forward_cell_updates = 0
        self.adjoint_cell_updates = 0
        self.makespan = 0.0

    # ---- job lifecycle on the device
    def _prepare(self, job: Job, stream=None) -> None:
        """Places an admitted job on the device and builds its plan (run by the placement
        worker, its uploads on ``stream``, which it drains before the job is handed over)."""
        from fdtdx_gb300.engine import Scene
        from fdtdx_gb300.fdtd import _materials_detached

        rec = job.kind == "gradient"
        st = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(st):
            job.objects, job.arrays, job.config = job.build("cuda", rec)
            job.state = _materials_detached(job.arrays).reset()
            job.scene = Scene(job.objects, job.state, job.config, record_interfaces=rec)
            job.scene.plan  # the plan's tables are built and uploaded here, off the loop thread
        st.synchronize()
        job.steps = job.config.time_steps_total

    def _batch_for(self, jobs: list[Job]):
        from fdtdx_gb300.batch import SimulationBatch

        key = tuple(j.id for j in jobs)
        if key == self._members and self._batch is not None:
            return self._batch, False
        if self._batch is not None:
            self._batch.close()
            self._batch = None
        self._members = key
        b = SimulationBatch([(j.state, j.objects, j.config) for j in jobs], scenes=[j.scene for j in jobs], reset=False)
        if self._tile is not None:
            b.tune(*self._tile[:4])
            b.set_mode(self._tile[4])
        self._batch = b
        return b, True

    def _start_adjoint(self, job: Job) -> None:
        st = job.state
        det = {n: {k: v.detach().clone().requires_grad_(True) for k, v in s.items()}
               for n, s in st.detector_states.items()}
        with torch.enable_grad():
            loss = job.loss(det)
            leaves = [v for s in det.values() for v in s.values()]
            grads = torch.autograd.grad(loss, leaves, allow_unused=True)
        job.loss_value = float(loss.detach())
        job.detectors = {n: {k: v.detach().clone() for k, v in s.items()} for n, s in st.detector_states.items()}
        lam_det, q = {}, 0
        for n, s in det.items():
            for _k, v in s.items():
                g = grads[q]
                q += 1
                if g is not None:
                    lam_det[n] = g.detach().contiguous()
        f = st.fields
        job.lam = {
            "E": torch.zeros_like(f.E), "H": torch.zeros_like(f.H),
            "psi_E": {k: (torch.zeros_like(a), torch.zeros_like(b)) for k, (a, b) in f.psi_E.items()},
            "psi_H": {k: (torch.zeros_like(a), torch.zeros_like(b)) for k, (a, b) in f.psi_H.items()},
            "det": lam_det,
            "grad_inv_eps": torch.zeros_like(st.inv_permittivities),
        }
        self.sched.start_adjoint(job)

    def cancel(self, job: Job) -> None:
        """Cancels a job: one not yet arrived is dropped when it arrives, a queued one leaves the
        queue, a running one stops at the next chunk boundary and releases its device state."""
        job.cancel_requested = True

    def snapshot(self, job: Job) -> dict:
        """Host copy of a running job's device state: the step it holds, E, H and the detector
        states (during the adjoint phase, the reconstructed state and its step).  Waits for
        the job's chunk in flight, if any."""
        if job.state is None:
            raise ValueError(f"job {job.id} holds no device state (phase {job.phase})")
        torch.cuda.synchronize()
        st = job.state
        t = job.t_fwd + job.inflight if job.phase == "forward" else job.t_adj - 1 - job.inflight
        return {"t": t, "phase": job.phase, "E": st.fields.E.detach().cpu(), "H": st.fields.H.detach().cpu(),
                "detectors": {n: {k: v.detach().cpu() for k, v in d.items()} for n, d in st.detector_states.items()}}

    def _release(self, job: Job, now: float, phase: str, error: str | None = None) -> None:
        """Ends a job without a result (cancelled or failed) and frees its device state."""
        if self._batch is not None and job.id in self._members:
            self._batch.close()  # it references the job's plan and buffers
            self._batch = None
            self._members = ()
        if job.scene is not None:
            job.scene.close()
        job.scene = job.state = job.arrays = job.lam = None
        job.error = error
        self.sched.complete(job, now, phase)

    def _diverged(self, job: Job) -> str | None:
        """The native finite check of the job's fields (E and H read once): the error message
        when they hold a NaN or an infinity, else None."""
        from fdtdx_gb300 import _native as N

        job.scene.forward(job.state, job.t_fwd, 0, graph=False, check_finite=True)
        try:
            job.scene.status()
        except N.NativeError as e:
            if e.code == N.ENONFINITE:
                return str(e)
            raise
        return None

    def _finish(self, job: Job, now: float) -> None:
        job.scene.status()
        if job.kind == "gradient":
            job.grad = job.lam["grad_inv_eps"] if self.keep_results else job.lam["grad_inv_eps"].cpu()
            job.lam = None
            job.state = None  # reconstructed back to the start: nothing to return
        elif self.keep_results:
            job.result = job.state
        else:
            job.detectors = {n: {k: v.detach().cpu() for k, v in st.items()} for n, st in job.state.detector_states.items()}
            job.state = None
        job.scene.close()
        job.scene = None
        job.arrays = None
        self.sched.complete(job, now)
        if job.footprint > 2**30:
            torch.cuda.empty_cache()  # hand large blocks back so the next large job can be placed

    # ---- the loop
    def run(self, jobs: list[Job], realtime: bool = True,
            on_chunk: Callable[["Server", float], None] | None = None) -> list[Job]:
        """Serve ``jobs`` (arrivals replayed in real time when ``realtime``, else idle gaps
        before an arrival are skipped); returns them done, cancelled or failed.

        The loop never waits for the whole device: the forward batch and every adjoint lane are
        polled through their CUDA events, and each gets its next chunk as soon as its last one
        has finished.  Admitted jobs are placed and their plans built by a worker thread on a
        side stream while the device runs the others.  ``on_chunk(server, now)`` runs after
        every finished chunk; ``cancel`` and ``snapshot`` may be called there.  A job whose
        fields turn non-finite fails alone (phase "failed", ``error`` set)."""
        import concurrent.futures as cf

        dev = torch.device("cuda")
        s_fwd = torch.cuda.Stream(dev)
        s_prep = torch.cuda.Stream(dev)
        lanes = [torch.cuda.Stream(dev) for _ in range(self.adjoint_lanes)]
        for i, j in enumerate(jobs):
            j.id = i
            if not j.footprint:
                estimate_footprint(j)
        pending = collections.deque(sorted(jobs, key=lambda j: j.arrival))
        t_start = time.perf_counter()
        skipped = [0.0]  # idle time jumped over when not replaying arrivals in real time

        def clock() -> float:
            return time.perf_counter() - t_start + skipped[0]

        pool = cf.ThreadPoolExecutor(max_workers=1, thread_name_prefix="fdtd-serve-prep")
        preparing: dict[int, cf.Future] = {}
        ready: set[int] = set()
        fwd = None              # in-flight forward chunk: (start event, end event, jobs, steps)
        adj: dict[int, tuple] = {}  # job id -> (lane, start event, end event, steps)
        lane_of: dict[int, int] = {}
        try:
            while pending or not self.sched.idle():
                progressed = False
                now = clock()
                while pending and pending[0].arrival <= now:
                    job = pending.popleft()
                    if job.cancel_requested:
                        job.phase, job.t_done = "cancelled", now
                        self.sched.done.append(job)
                        continue
                    self.sched.arrive(job)
                for job in list(self.sched.queue):
                    if job.cancel_requested:
                        self.sched.withdraw(job, now)
                for job in list(self.sched.active):
                    busy = job.id in adj or job.id in preparing or (fwd is not None and job in fwd[2])
                    if job.cancel_requested and not busy:
                        ready.discard(job.id)
                        self._release(job, now, "cancelled")
                for job in self.sched.admit(now):
                    preparing[job.id] = pool.submit(self._prepare, job, s_prep)
                for jid, fut in list(preparing.items()):
                    if fut.done():
                        fut.result()  # a placement error ends the loop with its exception
                        del preparing[jid]
                        ready.add(jid)
                        progressed = True
                # forward lane: account the finished chunk, issue the next one
                if fwd is not None and fwd[1].query():
                    self._forward_done(fwd, clock())
                    fwd = None
                    progressed = True
                if fwd is None:
                    fw = [j for j in self.sched.forward_jobs() if j.id in ready and not j.cancel_requested]
                    if fw:
                        fwd = self._issue_forward(fw, s_fwd)
                        progressed = True
                # adjoint lanes: one chunk per lane in flight
                for job in list(self.sched.adjoint_jobs()):
                    rec = adj.get(job.id)
                    if rec is not None and rec[2].query():
                        del adj[job.id]
                        self._adjoint_done(job, rec, clock())
                        progressed = True
                busy_lanes = {rec[0] for rec in adj.values()}
                for job in self.sched.adjoint_jobs():
                    if job.id in adj:
                        continue
                    if job.cancel_requested:
                        self._release(job, clock(), "cancelled")
                        progressed = True
                        continue
                    lane = lane_of.setdefault(job.id, len(lane_of) % len(lanes))
                    if lane in busy_lanes:
                        continue
                    adj[job.id] = self._issue_adjoint(job, lanes[lane], lane)
                    busy_lanes.add(lane)
                    progressed = True
                if progressed:
                    if on_chunk is not None:
                        on_chunk(self, clock())
                    continue
                if fwd is not None or adj:
                    time.sleep(2e-4)
                elif preparing:
                    cf.wait(list(preparing.values()), timeout=0.01, return_when=cf.FIRST_COMPLETED)
                elif pending:
                    wait = pending[0].arrival - clock()
                    if wait > 0:
                        if realtime:
                            time.sleep(min(wait, 0.01))
                        else:
                            skipped[0] += wait
        finally:
            pool.shutdown(wait=True)
            torch.cuda.synchronize()
            if self._batch is not None:
                self._batch.close()
                self._batch = None
                self._members = ()
        self.makespan = clock()
        return jobs

    def _issue_forward(self, fw: list[Job], stream) -> tuple:
        """One chunk of the forward batch of ``fw`` on ``stream`` (about target_chunk_s of work)."""
        cells = sum(j.cells for j in fw)
        cap = max(8, min(1000, int(self.target * self.rate / cells)))
        n = max(1, min(cap, min(j.steps - j.t_fwd for j in fw)))
        b, fresh = self._batch_for(fw)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            b.advance(n, t0=[j.t_fwd for j in fw] if fresh else None, graph=True,
                      autotune=self.autotune and self._tile is None, stream=stream)
            e1.record(stream)
        for j in fw:
            j.inflight = n
        return (e0, e1, fw, n)

    def _forward_done(self, rec: tuple, now: float) -> None:
        e0, e1, fw, n = rec
        ms = e0.elapsed_time(e1)
        cells = sum(j.cells for j in fw)
        if ms > 0:
            self.rate = 0.7 * self.rate + 0.3 * cells * n / (ms * 1e-3)
        if self._tile is None and self.autotune and self._batch is not None:
            t = self._batch.tuning()
            self._tile = (t["chunk_scale"][0], t["chunk_scale"][1], t["shell_chunk"], t["blocks_per_sm"], t["mode"])
        for j in fw:
            j.inflight = 0
            self.sched.advanced(j, n)
            self.forward_cell_updates += j.cells * n
            if j.cancel_requested:
                self._release(j, now, "cancelled")
            elif self.sched.forward_finished(j):
                err = self._diverged(j)
                if err is not None:
                    self._release(j, now, "failed", err)
                elif j.kind == "gradient":
                    self._start_adjoint(j)
                else:
                    self._finish(j, now)

    def _issue_adjoint(self, job: Job, stream, lane: int) -> tuple:
        """One chunk of ``job``'s adjoint loop on its lane's stream."""
        n = min(job.t_adj, max(8, int(self.target * self.adj_rate / job.cells)))
        stream.wait_stream(torch.cuda.current_stream())  # its cotangents were zeroed there
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            job.scene.adjoint(job.state, job.lam, job.t_adj - 1, n, stream=stream)
            e1.record(stream)
        job.inflight = n
        return (lane, e0, e1, n)

    def _adjoint_done(self, job: Job, rec: tuple, now: float) -> None:
        _lane, e0, e1, n = rec
        ms = e0.elapsed_time(e1)
        if ms > 0:
            self.adj_rate = 0.7 * self.adj_rate + 0.3 * job.cells * n / (ms * 1e-3)
        job.inflight = 0
        job.t_adj -= n
        self.adjoint_cell_updates += job.cells * n
        if job.cancel_requested:
            self._release(job, now, "cancelled")
        elif job.t_adj <= 0:
            self._finish(job, now)


def run_one_at_a_time(jobs: list[Job], realtime: bool = True, keep_results: bool = True) -> list[Job]:
    """The plain path: each job alone through run_fdtd / reversible_fdtd, in arrival order.
    ``keep_results=False`` keeps only the host copies of the detector states (and gradients)."""
    from fdtdx_gb300.adjoint import reversible_fdtd
    from fdtdx_gb300.fdtd import run_fdtd

    t0 = time.perf_counter()
    for i, j in enumerate(sorted(jobs, key=lambda j: j.arrival)):
        j.id = i
        if realtime:
            wait = j.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        j.t_admit = time.perf_counter() - t0
        objects, arrays, config = j.build("cuda", j.kind == "gradient")
        j.steps = config.time_steps_total
        n = objects.volume.grid_shape
        j.n_cells = n[0] * n[1] * n[2]
        if j.kind == "gradient":
            ie = arrays.inv_permittivities.detach().clone().requires_grad_(True)
            _, out = reversible_fdtd(arrays.aset("inv_permittivities", ie), objects, config)
            loss = j.loss(out.detector_states)
            (g,) = torch.autograd.grad(loss, [ie])
            j.grad, j.loss_value = g.detach(), float(loss.detach())
            j.detectors = {dn: {k: v.detach().clone() for k, v in st.items()} for dn, st in out.detector_states.items()}
            if not keep_results:
                j.grad = j.grad.cpu()
                j.detectors = {dn: {k: v.cpu() for k, v in st.items()} for dn, st in j.detectors.items()}
            del out, ie, g, loss
        else:
            _, res = run_fdtd(arrays, objects, config)
            if keep_results:
                j.result = res
            else:
                j.detectors = {dn: {k: v.detach().cpu() for k, v in st.items()} for dn, st in res.detector_states.items()}
            del res
        torch.cuda.synchronize()
        j.t_done = time.perf_counter() - t0
        j.phase = "done"
        del objects, arrays
        if not keep_results and j.footprint > 2**30:
            torch.cuda.empty_cache()
    return jobs


def latency_stats(jobs: list[Job]) -> dict:
    lat = sorted(j.latency for j in jobs)
    if not lat:
        return {"p50_s": None, "p99_s": None, "mean_s": None}

    def pct(p):
        k = min(len(lat) - 1, max(0, int(math.ceil(p / 100.0 * len(lat))) - 1))
        return lat[k]

    return {"p50_s": pct(50), "p99_s": pct(99), "mean_s": sum(lat) / len(lat)}
