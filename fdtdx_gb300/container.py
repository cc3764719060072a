"""State containers with fdtdx's field names (fdtdx/fdtd/container.py:33-495).

``ArrayContainer`` holds torch tensors (device memory on the GPU path):

* ``fields.E`` / ``fields.H``           (3, nx, ny, nz) float32
* ``fields.psi_E`` / ``fields.psi_H``   {pml name: (psi_1, psi_2)}, each ``pml.grid_shape``
* ``inv_permittivities``                (1|3|9, nx, ny, nz) (9: a row-major full tensor)
* ``inv_permeabilities``                float 1.0 (non-magnetic) or (1|3|9, nx, ny, nz)
* ``electric_conductivity`` / ``magnetic_conductivity``  None or (1|3|9, nx, ny, nz), pre-scaled by dx
* ``fields.dispersive_P_curr`` / ``_P_prev``  None or (poles, 3, nx, ny, nz): the ADE polarisation
* ``dispersive_c1`` / ``_c2`` / ``_c3``  None or (poles, 1|3, nx, ny, nz): its recurrence coefficients
* ``detector_states``                   {detector name: {key: tensor}}
* ``recording_state``                   None or ``RecordingState`` of the PML-interface recorder
"""

from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import Any

import torch

from fdtdx_gb300.objects import (
    BaseBoundary,
    Detector,
    Device,
    PerfectlyMatchedLayer,
    SimulationObject,
    SimulationVolume,
    Source,
    UniformMaterialObject,
)

PmlAuxField = dict[str, tuple[torch.Tensor, torch.Tensor]]


@dataclass
class RecordingState:
    """Recorded PML-interface planes: ``data["interfaces"]`` is (T, floats per step) in the storage dtype."""

    data: dict[str, torch.Tensor]
    state: dict[str, torch.Tensor] = field(default_factory=dict)


def _aset(obj, path: str, value):
    parts = path.split("->")
    if len(parts) == 1:
        return dataclasses.replace(obj, **{parts[0]: value})
    head = getattr(obj, parts[0])
    return dataclasses.replace(obj, **{parts[0]: _aset(head, "->".join(parts[1:]), value)})


@dataclass
class FieldState:
    E: torch.Tensor
    H: torch.Tensor
    psi_E: PmlAuxField
    psi_H: PmlAuxField
    dispersive_P_curr: torch.Tensor | None = None
    dispersive_P_prev: torch.Tensor | None = None

    def aset(self, path: str, value) -> "FieldState":
        return _aset(self, path, value)


@dataclass
class ArrayContainer:
    fields: FieldState
    inv_permittivities: torch.Tensor
    inv_permeabilities: torch.Tensor | float
    detector_states: dict[str, dict[str, torch.Tensor]]
    recording_state: RecordingState | None
    electric_conductivity: torch.Tensor | None = None
    magnetic_conductivity: torch.Tensor | None = None
    initial_inv_permittivities: torch.Tensor | None = None
    dispersive_c1: torch.Tensor | None = None
    dispersive_c2: torch.Tensor | None = None
    dispersive_c3: torch.Tensor | None = None
    dispersive_c4: torch.Tensor | None = None

    def aset(self, path: str, value) -> "ArrayContainer":
        """Functional update, ``arrays.aset("fields->E", E)`` as in fdtdx."""
        return _aset(self, path, value)

    def reset(self, reset_detector_states: bool = True, reset_recording_state: bool = False) -> "ArrayContainer":
        """Zero the fields and psi (and detector states); keep materials (container.py:451-491)."""
        f = self.fields
        fields = FieldState(
            E=torch.zeros_like(f.E),
            H=torch.zeros_like(f.H),
            psi_E={k: (torch.zeros_like(a), torch.zeros_like(b)) for k, (a, b) in f.psi_E.items()},
            psi_H={k: (torch.zeros_like(a), torch.zeros_like(b)) for k, (a, b) in f.psi_H.items()},
            dispersive_P_curr=None if f.dispersive_P_curr is None else torch.zeros_like(f.dispersive_P_curr),
            dispersive_P_prev=None if f.dispersive_P_prev is None else torch.zeros_like(f.dispersive_P_prev),
        )
        det = self.detector_states
        if reset_detector_states:
            det = {k: {k2: torch.zeros_like(v2) for k2, v2 in v.items()} for k, v in det.items()}
        rec = self.recording_state
        if reset_recording_state and rec is not None:
            rec = RecordingState({k: torch.zeros_like(v) for k, v in rec.data.items()},
                                 {k: torch.zeros_like(v) for k, v in rec.state.items()})
        return dataclasses.replace(self, fields=fields, detector_states=det, recording_state=rec)

    @property
    def device(self) -> torch.device:
        return self.fields.E.device


@dataclass
class ObjectContainer:
    """The placed simulation objects (fdtdx/fdtd/container.py:33-355)."""

    object_list: list[SimulationObject]
    volume_idx: int = 0

    @property
    def volume(self) -> SimulationVolume:
        return self.object_list[self.volume_idx]  # type: ignore[return-value]

    @property
    def objects(self) -> list[SimulationObject]:
        return self.object_list

    @property
    def sources(self) -> list[Source]:
        return [o for o in self.object_list if isinstance(o, Source)]

    @property
    def detectors(self) -> list[Detector]:
        return [o for o in self.object_list if isinstance(o, Detector)]

    @property
    def forward_detectors(self) -> list[Detector]:
        return [d for d in self.detectors if not d.inverse]

    @property
    def backward_detectors(self) -> list[Detector]:
        return [d for d in self.detectors if d.inverse]

    @property
    def pml_objects(self) -> list[PerfectlyMatchedLayer]:
        return [o for o in self.object_list if isinstance(o, PerfectlyMatchedLayer)]

    @property
    def boundary_objects(self) -> list[BaseBoundary]:
        return [o for o in self.object_list if isinstance(o, BaseBoundary)]

    @property
    def static_material_objects(self) -> list[UniformMaterialObject]:
        return [o for o in self.object_list if isinstance(o, UniformMaterialObject)]

    @property
    def devices(self) -> list[Device]:
        return [o for o in self.object_list if isinstance(o, Device)]

    def __getitem__(self, name: str) -> SimulationObject:
        for o in self.object_list:
            if o.name == name:
                return o
        raise KeyError(name)


ParameterContainer = dict[str, torch.Tensor]
SimulationState = tuple[int, ArrayContainer]
Info = dict[str, Any]
