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


class Recorder:
    """Records the PML-interface planes of E and H after every forward step.

    fdtdx/interfaces/recorder.py:14-199.  The identity recorder (no modules) keeps
    float32 planes; a ``DtypeConversion`` module narrows the storage.
    """

    def __init__(self, modules: Sequence[object] = ()):
        self.modules = list(modules)
        for m in self.modules:
            if not isinstance(m, DtypeConversion):
                raise NotImplementedError(f"recorder module {type(m).__name__} is not supported")

    @property
    def storage_dtype(self) -> torch.dtype:
        dt = torch.float32
        for m in self.modules:
            dt = m.dtype
        return dt


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
