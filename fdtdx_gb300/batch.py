"""Batched forward runs: many simulations stepped together on the native batch path.

There is no batch API in fdtdx (a user loops ``run_fdtd`` over simulations); this is
the GB300 replacement for that loop.  Every simulation keeps its own plan and buffers;
``fdtd_batch_forward`` advances all of them with one persistent launch per kernel kind
and step, replayed from a CUDA graph, with tile shapes chosen by the native online
autotuner.  Results equal the per-simulation path (the same device code runs per block).
"""

from __future__ import annotations

import ctypes as C
from typing import Sequence

import torch

from fdtdx_gb300 import _native as N
from fdtdx_gb300.config import SimulationConfig
from fdtdx_gb300.container import ArrayContainer, ObjectContainer, SimulationState
from fdtdx_gb300.engine import Scene


class SimulationBatch:
    """A set of forward simulations (uneven grids allowed) advanced together.

    ``sims`` holds ``(arrays, objects, config)`` triples as ``run_fdtd`` takes them.  The
    batch owns reset copies of the arrays; ``results()`` returns them as
    ``(time_step, arrays)`` pairs.
    """

    def __init__(self, sims: Sequence[tuple[ArrayContainer, ObjectContainer, SimulationConfig]],
                 scenes: Sequence[Scene] | None = None, reset: bool = True):
        """``scenes`` (optional) are already-built scenes of the simulations (e.g. recording
        ones for gradient jobs); ``reset=False`` steps the given arrays in place."""
        from fdtdx_gb300.fdtd import _materials_detached

        if not sims:
            raise ValueError("a batch needs at least one simulation")
        self.scenes: list[Scene] = []
        self.arrays: list[ArrayContainer] = []
        self.configs: list[SimulationConfig] = []
        self._own_scenes = scenes is None
        for q, (arrays, objects, config) in enumerate(sims):
            work = _materials_detached(arrays).reset() if reset else arrays
            self.scenes.append(Scene(objects, work, config, record_interfaces=False) if scenes is None else scenes[q])
            self.arrays.append(work)
            self.configs.append(config)
        n = len(self.scenes)
        lib = N.load()
        plans = (C.c_void_p * n)(*[s.plan for s in self.scenes])
        self._bufs = (N.Buffers * n)(*[s.buffers(a) for s, a in zip(self.scenes, self.arrays)])
        h = C.c_void_p()
        N.check(lib.fdtd_batch_create(plans, self._bufs, n, C.byref(h)), None, "fdtd_batch_create")
        self._h = h.value
        self.t = [0] * n

    def _check(self, rc: int, what: str) -> None:
        if rc != N.OK:
            msg = N.load().fdtd_batch_last_error(self._h)
            raise N.NativeError(f"{what}: {rc} {msg.decode() if msg else ''}", rc)

    def advance(self, n_steps: int, t0: Sequence[int] | None = None, graph: bool = True, autotune: bool = True,
                stream=None) -> None:
        """Advance every simulation by ``n_steps`` (from ``t0`` when given)."""
        st = stream if stream is not None else torch.cuda.current_stream(self.arrays[0].device)
        ts = None
        if t0 is not None:
            ts = (C.c_int32 * len(self.scenes))(*[int(x) for x in t0])
            self.t = [int(x) for x in t0]
        flags = (1 if graph else 0) | (2 if autotune else 0)
        rc = N.load().fdtd_batch_forward(self._h, ts, int(n_steps), flags, C.c_void_p(st.cuda_stream))
        self._check(rc, "fdtd_batch_forward")
        self.t = [x + int(n_steps) for x in self.t]

    def run(self, graph: bool = True, autotune: bool = True) -> list[SimulationState]:
        """Run every simulation for its ``time_steps_total`` (all must be equal) from step 0."""
        Ts = {c.time_steps_total for c in self.configs}
        if len(Ts) != 1:
            raise ValueError("run() needs equal step counts; use advance() for uneven ones")
        T = Ts.pop()
        self.advance(T, t0=[0] * len(self.scenes), graph=graph, autotune=autotune)
        for s in self.scenes:
            s.status()
        return self.results()

    def results(self) -> list[SimulationState]:
        return [(t, a) for t, a in zip(self.t, self.arrays)]

    def tuning(self) -> dict:
        out = (C.c_int32 * 4)()
        self._check(N.load().fdtd_batch_tuning(self._h, out), "fdtd_batch_tuning")
        return {"chunk_scale": (out[0], out[1]), "shell_chunk": out[2], "blocks_per_sm": out[3], "mode": self.mode}

    def tune(self, chunk_num: int = 1, chunk_den: int = 1, shell_chunk: int = 4, blocks_per_sm: int = 8) -> None:
        rc = N.load().fdtd_batch_tune(self._h, chunk_num, chunk_den, shell_chunk, blocks_per_sm)
        self._check(rc, "fdtd_batch_tune")

    @property
    def mode(self) -> str:
        return {0: "persistent", 1: "branches", 2: "fused"}[int(N.load().fdtd_batch_mode(self._h))]

    def set_mode(self, mode: str) -> None:
        rc = N.load().fdtd_batch_set_mode(self._h, {"persistent": 0, "branches": 1, "fused": 2}[mode])
        self._check(rc, "fdtd_batch_set_mode")

    def launches_per_step(self) -> int:
        return int(N.load().fdtd_batch_launches_per_step(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.load().fdtd_batch_destroy(self._h)
            self._h = None
        if getattr(self, "_own_scenes", False):
            for s in self.scenes:
                s.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_fdtd_batch(sims: Sequence[tuple[ArrayContainer, ObjectContainer, SimulationConfig]],
                   autotune: bool = True) -> list[SimulationState]:
    """``run_fdtd`` over many forward simulations at once; returns one ``(T, arrays)`` each."""
    batch = SimulationBatch(sims)
    try:
        return batch.run(autotune=autotune)
    finally:
        batch.close()
