"""Scene placement and array initialisation (host setup, run once per simulation).

Restates what the time-stepping path consumes from fdtdx/fdtd/initialization.py:
array shapes and dtypes (``_init_arrays``, :552-1205), material painting in
``placement_order`` (:844-930, conductivity scaled by the grid spacing :784-786),
detector state shapes (detector.py:231-244 and the ``_shape_dtype_single_time_step``
of each detector) and the continuous device mapping of ``apply_params``
(:404-417).  Objects are placed by their explicit ``grid_slice_tuple``; the
reference's constraint solver is not part of this package.
"""

from __future__ import annotations

import dataclasses
from typing import Sequence

import numpy as np
import torch

from fdtdx_gb300.config import SimulationConfig
from fdtdx_gb300.container import ArrayContainer, FieldState, ObjectContainer, ParameterContainer, RecordingState
from fdtdx_gb300.objects import (
    Detector,
    Device,
    EnergyDetector,
    FieldDetector,
    Material,
    PhasorDetector,
    PoyntingFluxDetector,
    SimulationObject,
    SimulationVolume,
    UniformMaterialObject,
)


def _default_device() -> torch.device:
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


def detector_state_shapes(det: Detector, config: SimulationConfig) -> dict[str, tuple[tuple[int, ...], torch.dtype]]:
    """Per-detector state keys, shapes and dtypes (the reference's ``init_state``)."""
    gs = det.grid_shape
    if isinstance(det, PhasorDetector):
        F, C = len(det.wave_characters), len(det.recorded_components)
        shape = (1, F, C) if det.reduce_volume else (1, F, C, *gs)
        return {"phasor": (shape, torch.complex64)}
    T_on = det.num_time_steps_recorded(config)
    if isinstance(det, FieldDetector):
        C = len(det.recorded_components)
        return {"fields": ((T_on, C) if det.reduce_volume else (T_on, C, *gs), torch.float32)}
    if isinstance(det, PoyntingFluxDetector):
        if det.keep_all_components:
            shape = (T_on, 3) if det.reduce_volume else (T_on, 3, *gs)
        else:
            shape = (T_on, 1) if det.reduce_volume else (T_on, *gs)
        return {"poynting_flux": (shape, torch.float32)}
    if isinstance(det, EnergyDetector):
        return {"energy": ((T_on, 1) if det.reduce_volume else (T_on, *gs), torch.float32)}
    raise NotImplementedError(f"detector type {type(det).__name__} is not supported")


def _n_components(materials: Sequence[Material], attr: str) -> int:
    """1 (isotropic), 3 (diagonal) or 9 (a full tensor somewhere) components for ``attr``
    (fdtdx/fdtd/initialization.py:552-620 picks the array width the same way)."""
    vals = [getattr(m, attr) for m in materials]
    if all(Material._iso(v) for v in vals):
        return 1
    if all(Material._diag(v) for v in vals):
        return 3
    return 9


def _comp_values(t9, n: int) -> list[float]:
    if n == 9:
        return list(t9)
    return [t9[0]] if n == 1 else [t9[0], t9[4], t9[8]]


def _inverse_values(t9, n: int) -> list[float]:
    """The stored inverse of a permittivity / permeability: elementwise for 1 or 3 components,
    the matrix inverse of the row-major tensor for 9 (initialization.py:866-877, 2145-2161)."""
    if n == 9:
        return [float(x) for x in np.linalg.inv(np.asarray(t9, dtype=np.float64).reshape(3, 3)).reshape(9)]
    return [1.0 / v for v in _comp_values(t9, n)]


def dispersive_coefficients(objects: ObjectContainer, config: SimulationConfig):
    """Per-cell ADE recurrence coefficients (c1, c2, c3), each (poles, 1 | 3, nx, ny, nz) float32,
    or None without a dispersive material (fdtdx/fdtd/initialization.py:686-700, 795-830,
    955-1000): every painted material, the volume first, then the material objects in placement
    order, writes its pole stack over its slice, zero-padded to the scene's largest pole count
    (all zeros for a material without poles); one component when every pole is isotropic, else
    three.  Coefficients of fdtdx/dispersion.py:789-857."""
    from fdtdx_gb300.dispersion import compute_pole_coefficients_per_axis

    painted = [objects.volume] + sorted(objects.static_material_objects, key=lambda o: o.placement_order)
    models = [o.material.dispersion for o in painted
              if o.material is not None and o.material.dispersion is not None and o.material.dispersion.num_poles > 0]
    if not models:
        return None
    n_poles = max(m.num_poles for m in models)
    nc = 1 if all(m.is_isotropic for m in models) else 3
    shape = objects.volume.grid_shape
    dt = config.time_step_duration
    out = [torch.zeros((n_poles, nc, *shape), dtype=torch.float32) for _ in range(3)]
    for o in painted:
        if o.material is None:
            continue
        block = [np.zeros((n_poles, nc)) for _ in range(3)]
        disp = o.material.dispersion
        if disp is not None and disp.num_poles > 0:
            for pole in disp.poles:
                if getattr(pole, "orientation", None) is not None:
                    raise NotImplementedError("oriented dispersive poles are not supported")
            cs = compute_pole_coefficients_per_axis(disp.poles, dt)
            for q in range(3):
                block[q][: disp.num_poles] = cs[q][:, :nc]
        sl = (slice(None), slice(None), *o.grid_slice)
        for q in range(3):
            out[q][sl] = torch.tensor(block[q], dtype=torch.float32)[:, :, None, None, None]
    return tuple(out)


def init_arrays(objects: ObjectContainer, config: SimulationConfig, device=None) -> ArrayContainer:
    """Allocate and fill the ArrayContainer of a placed scene."""
    device = torch.device(device) if device is not None else _default_device()
    shape = objects.volume.grid_shape
    N3 = (3, *shape)
    # complex fields exactly when a Bloch boundary carries a non-zero vector component
    # (fdtdx/fdtd/initialization.py:581-594)
    complex_fields = any(getattr(b, "needs_complex_fields", False) for b in objects.boundary_objects)
    fdt = torch.complex64 if complex_fields else torch.float32
    E = torch.zeros(N3, dtype=fdt, device=device)
    H = torch.zeros(N3, dtype=fdt, device=device)
    psi_E = {p.name: (torch.zeros(p.grid_shape, dtype=fdt, device=device),
                      torch.zeros(p.grid_shape, dtype=fdt, device=device)) for p in objects.pml_objects}
    psi_H = {p.name: (torch.zeros(p.grid_shape, dtype=fdt, device=device),
                      torch.zeros(p.grid_shape, dtype=fdt, device=device)) for p in objects.pml_objects}

    vol = objects.volume
    bg = vol.material if vol.material is not None else Material()
    painted: list[tuple[SimulationObject, Material]] = [(vol, bg)]
    mats = sorted(objects.static_material_objects, key=lambda o: o.placement_order)
    painted += [(o, o.material) for o in mats]
    dev_objs = objects.devices
    dev_mats = [Material(permittivity=d.permittivity_low) for d in dev_objs] + [
        Material(permittivity=d.permittivity_high) for d in dev_objs
    ]
    all_mats = [m for _, m in painted] + dev_mats
    n_eps = _n_components(all_mats, "permittivity")
    n_mu = _n_components(all_mats, "permeability")
    magnetic = any(m.is_magnetic for m in all_mats)
    econd = any(m.is_electrically_conductive for m in all_mats)
    mcond = any(m.is_magnetically_conductive for m in all_mats)
    n_se = _n_components(all_mats, "electric_conductivity") if econd else 0
    n_sh = _n_components(all_mats, "magnetic_conductivity") if mcond else 0
    spacing = config.uniform_spacing()

    inv_eps = torch.zeros((n_eps, *shape), dtype=torch.float32)
    inv_mu = torch.zeros((n_mu, *shape), dtype=torch.float32) if magnetic else None
    sig_e = torch.zeros((n_se, *shape), dtype=torch.float32) if econd else None
    sig_h = torch.zeros((n_sh, *shape), dtype=torch.float32) if mcond else None
    for o, m in painted:
        sl = (slice(None), *o.grid_slice)
        inv_eps[sl] = torch.tensor(_inverse_values(m.permittivity, n_eps), dtype=torch.float32)[:, None, None, None]
        if inv_mu is not None:
            inv_mu[sl] = torch.tensor(_inverse_values(m.permeability, n_mu), dtype=torch.float32)[:, None, None, None]
        if sig_e is not None:
            sig_e[sl] = (torch.tensor(_comp_values(m.electric_conductivity, n_se), dtype=torch.float32) * spacing)[
                :, None, None, None]
        if sig_h is not None:
            sig_h[sl] = (torch.tensor(_comp_values(m.magnetic_conductivity, n_sh), dtype=torch.float32) * spacing)[
                :, None, None, None]

    det_states = {}
    for d in objects.detectors:
        det_states[d.name] = {
            k: torch.zeros(shp, dtype=dt, device=device) for k, (shp, dt) in detector_state_shapes(d, config).items()
        }

    rec = None
    gc = config.gradient_config
    if gc is not None and gc.recorder is not None:
        per_step = 6 * sum(int(torch.tensor(p.grid_shape).prod()) // p.thickness for p in objects.pml_objects)
        rdt = gc.recorder.storage_dtype
        if complex_fields:
            if rdt != torch.float32:
                raise NotImplementedError("complex (Bloch) fields are recorded in float32 only")
            rdt = torch.complex64
        data = torch.zeros((gc.recorder.slots(config.time_steps_total), per_step), dtype=rdt, device=device)
        rec = RecordingState(data={"interfaces": data})

    disp = dispersive_coefficients(objects, config)
    P_curr = P_prev = None
    if disp is not None:
        P_curr = torch.zeros((disp[0].shape[0], *N3), dtype=fdt, device=device)
        P_prev = torch.zeros_like(P_curr)
    return ArrayContainer(
        fields=FieldState(E=E, H=H, psi_E=psi_E, psi_H=psi_H, dispersive_P_curr=P_curr, dispersive_P_prev=P_prev),
        inv_permittivities=inv_eps.to(device),
        inv_permeabilities=inv_mu.to(device) if inv_mu is not None else 1.0,
        detector_states=det_states,
        recording_state=rec,
        electric_conductivity=sig_e.to(device) if sig_e is not None else None,
        magnetic_conductivity=sig_h.to(device) if sig_h is not None else None,
        dispersive_c1=None if disp is None else disp[0].to(device),
        dispersive_c2=None if disp is None else disp[1].to(device),
        dispersive_c3=None if disp is None else disp[2].to(device),
    )


def place_objects(
    object_list: Sequence[SimulationObject],
    config: SimulationConfig,
    constraints: Sequence = (),
    key=None,
    device=None,
) -> tuple[ObjectContainer, ArrayContainer, ParameterContainer, SimulationConfig, dict]:
    """Place objects by their ``grid_slice_tuple`` and initialise the arrays.

    Same return tuple as fdtdx's ``place_objects`` (fdtdx/fdtd/initialization.py:100-314):
    ``(objects, arrays, params, config, info)``.  Device parameters start at 0.5.
    """
    if constraints:
        raise NotImplementedError("constraint-based placement is not supported; give every object a grid_slice_tuple")
    del key
    vols = [i for i, o in enumerate(object_list) if isinstance(o, SimulationVolume)]
    if len(vols) != 1:
        raise ValueError("exactly one SimulationVolume is required")
    names = set()
    for idx, o in enumerate(object_list):
        if o.name is None:
            o.name = f"{type(o).__name__}_{idx}"
        if o.name in names:
            raise ValueError(f"duplicate object name {o.name}")
        names.add(o.name)
        if o.grid_slice_tuple is None:
            raise ValueError(f"object {o.name} has no grid_slice_tuple")
        shape = object_list[vols[0]].grid_shape
        for a, (lo, hi) in enumerate(o.grid_slice_tuple):
            if lo < 0 or hi > shape[a]:
                raise ValueError(f"object {o.name} lies outside the volume on axis {a}")
    objects = ObjectContainer(object_list=list(object_list), volume_idx=vols[0])
    arrays = init_arrays(objects, config, device=device)
    params: ParameterContainer = {
        d.name: torch.full(d.grid_shape, 0.5, dtype=torch.float32, device=arrays.device) for d in objects.devices
    }
    if objects.devices:
        arrays, objects, _ = apply_params(arrays, objects, params)
    return objects, arrays, params, config, {}


def apply_params(arrays: ArrayContainer, objects: ObjectContainer, params: ParameterContainer,
                 key=None) -> tuple[ArrayContainer, ObjectContainer, dict]:
    """Map device parameters to inv_eps: eps = eps_lo + p (eps_hi - eps_lo) (initialization.py:317-417).

    Returns ``(arrays, objects, info)`` like the reference.  Out-of-place, so a ``params``
    tensor with ``requires_grad`` carries the gradient.
    """
    del key
    inv = arrays.inv_permittivities.clone()
    for d in objects.devices:
        p = params[d.name]
        eps = d.permittivity_low + p * (d.permittivity_high - d.permittivity_low)
        if inv.shape[0] == 9:  # an isotropic device inside a full-tensor array: diag(1 / eps)
            z = torch.zeros_like(eps)
            inv[(slice(None), *d.grid_slice)] = torch.stack([1.0 / eps if q % 4 == 0 else z for q in range(9)])
        else:
            inv[(slice(None), *d.grid_slice)] = (1.0 / eps)[None].expand(inv.shape[0], *p.shape)
    return dataclasses.replace(arrays, inv_permittivities=inv), objects, {}
