"""Simulation and gradient configuration (fdtdx/config.py:15-307, fdtdx/core/grid.py UniformGrid).

Only the uniform Cartesian grid is supported: every kernel assumes one spacing
``dx`` on all three axes, which is what the reference's ``UniformGrid`` and a
uniform ``RectilinearGrid`` reduce to (``_metric_scale`` returns 1.0,
fdtdx/core/physics/curl.py:10-39).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Literal, Sequence

import torch

from fdtdx_gb300 import constants


@dataclass(frozen=True)
class UniformGrid:
    """Uniform spacing on all axes, in metres."""

    spacing: float


class DtypeConversion:
    """Interface-recorder compression stage that stores the recorded planes in a narrower dtype.

    fdtdx/interfaces/modules.py:99-161.  Supported storage types: ``torch.bfloat16`` and
    ``torch.float16`` (the reference's default is ``jnp.bfloat16``).
    """

    def __init__(self, dtype: torch.dtype = torch.bfloat16, exclude_filter: Sequence[str] = ()):
        if dtype not in (torch.bfloat16, torch.float16, torch.float32):
            raise ValueError(f"unsupported recorder storage dtype {dtype}")
        self.dtype = dtype
        self.exclude_filter = tuple(exclude_filter)


class LinearReconstructEveryK:
    """Interface-recorder time filter: store every k-th step, interpolate linearly between.

    fdtdx/interfaces/time_filter.py:140-257.  The stored steps are ``start_recording_after``,
    then every ``k`` steps, plus the last step T-1.  A stored step reads its own slot; any
    other step t reads ``prev + f * (next - prev)`` between the slot a at or before t and
    slot a + 1, with f = (t - t_a) / (t_{a+1} - t_a) and t_a the first step mapped to slot a.
    """

    def __init__(self, k: int, start_recording_after: int = 0):
        if k < 1:
            raise ValueError("k must be >= 1")
        self.k = int(k)
        self.start_recording_after = int(start_recording_after)

    def save_steps(self, T: int) -> list[int]:
        steps = list(range(self.start_recording_after, T, self.k))
        if not steps or steps[-1] != T - 1:
            steps.append(T - 1)
        return steps

    def time_to_slot(self, T: int) -> list[int]:
        """Slot of the last stored step at or before t (time_filter.py:180-191)."""
        idx = [0] * T
        for a, t in enumerate(self.save_steps(T)):
            idx[t] = a
        for _ in range(self.k - 1):  # each pass copies a slot one step to the right
            rolled = [idx[-1]] + idx[:-1]
            idx = [r if v == 0 else v for v, r in zip(idx, rolled)]
            for t in range(min(self.k, T)):
                idx[t] = 0
        return idx

    def tables(self, T: int) -> tuple[list[int], list[int], list[int], list[float]]:
        """Per step t = -1 .. T (entry t + 1): store slot (-1: not stored), and the restore
        slots a, b and weight w of ``v = v_a + w (v_b - v_a)``."""
        S = self.save_steps(T)
        Sset = set(S)
        m = self.time_to_slot(T)
        first = {}
        for t, a in enumerate(m):
            first.setdefault(a, t)
        A = len(S)
        store, sa, sb, w = [], [], [], []
        for t in range(-1, T + 1):
            tj = min(max(t + T if t < 0 else t, 0), T - 1)  # a JAX gather: -1 wraps, T clamps
            store.append(m[tj] if t in Sset else -1)
            a = m[tj]
            if tj in Sset:
                sa.append(a), sb.append(a), w.append(0.0)
                continue
            b = min(a + 1, A - 1)
            t_prev = first.get(a, 0)
            t_next = first.get(a + 1, 0)  # no step maps to a + 1: the first index (argmax of no match)
            f = (t - t_prev) / (t_next - t_prev) if t_next != t_prev else 0.0
            sa.append(a), sb.append(b), w.append(f)
        return store, sa, sb, w


class Recorder:
    """Records the PML-interface planes of E and H after every forward step.

    fdtdx/interfaces/recorder.py:14-199.  The identity recorder (no modules) keeps
    float32 planes; a ``DtypeConversion`` module narrows the storage; a
    ``LinearReconstructEveryK`` time filter stores every k-th step only.
    """

    def __init__(self, modules: Sequence[object] = ()):
        self.modules = list(modules)
        for m in self.modules:
            if not isinstance(m, (DtypeConversion, LinearReconstructEveryK)):
                raise NotImplementedError(f"recorder module {type(m).__name__} is not supported")
        if sum(isinstance(m, LinearReconstructEveryK) for m in self.modules) > 1:
            raise NotImplementedError("at most one time filter per recorder")

    @property
    def storage_dtype(self) -> torch.dtype:
        dt = torch.float32
        for m in self.modules:
            if isinstance(m, DtypeConversion):
                dt = m.dtype
        return dt

    @property
    def time_filter(self) -> LinearReconstructEveryK | None:
        for m in self.modules:
            if isinstance(m, LinearReconstructEveryK):
                return m
        return None

    def slots(self, T: int) -> int:
        """Recording rows for a run of T steps."""
        tf = self.time_filter
        return T if tf is None else len(tf.save_steps(T))


@dataclass
class GradientConfig:
    """How gradients are computed: ``"reversible"`` (time reversal + recorder) or ``"checkpointed"``."""

    method: Literal["reversible", "checkpointed"] = "reversible"
    recorder: Recorder | None = None
    num_checkpoints: int | None = None
    num_checkpoints_reversible: int = 0

    def __post_init__(self):
        if self.method == "reversible" and self.recorder is None:
            raise Exception("Need Recorder in gradient config to compute reversible gradients")
        if self.method == "checkpointed" and self.num_checkpoints is None:
            raise Exception("Need Checkpoint Number in gradient config to compute checkpointed gradients")
        if self.num_checkpoints_reversible < 0:
            raise Exception("num_checkpoints_reversible must be >= 0")


@dataclass
class SimulationConfig:
    """Time, grid, dtype and Courant settings of one simulation."""

    time: float
    grid: UniformGrid
    backend: str = "gpu"
    dtype: torch.dtype = torch.float32
    courant_factor: float = 0.99
    gradient_config: GradientConfig | None = None
    symmetry: tuple[int, int, int] = field(default=(0, 0, 0))

    def __post_init__(self):
        if self.dtype != torch.float32:
            raise NotImplementedError("the GB300 kernels compute in float32 only")
        if any(s != 0 for s in self.symmetry):
            raise NotImplementedError("symmetry domain reduction is not supported")

    @property
    def courant_number(self) -> float:
        return self.courant_factor / math.sqrt(3)

    def uniform_spacing(self) -> float:
        return self.grid.spacing

    @property
    def resolution(self) -> float:
        return self.grid.spacing

    @property
    def time_step_duration(self) -> float:
        return self.courant_number * self.grid.spacing / constants.c

    @property
    def time_steps_total(self) -> int:
        return round(self.time / self.time_step_duration)

    @property
    def only_forward(self) -> bool:
        return self.gradient_config is None

    @property
    def invertible_optimization(self) -> bool:
        return self.gradient_config is not None and self.gradient_config.recorder is not None
