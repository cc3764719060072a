"""Public drivers with fdtdx's signatures (fdtdx/fdtd/wrapper.py:14-63, fdtdx/fdtd/fdtd.py:39-496).

``run_fdtd`` dispatches on ``config.gradient_config`` exactly as the reference does.
The time loop runs in the native library (CUDA-graph replayed chunks of steps);
the Python side only builds the plan once per scene and hands over buffers.
"""

from __future__ import annotations

import warnings
from typing import Callable

import torch

from fdtdx_gb300.config import SimulationConfig
from fdtdx_gb300.container import ArrayContainer, ObjectContainer, SimulationState
from fdtdx_gb300.engine import Scene
from fdtdx_gb300.objects import LinearlyPolarizedPlaneSource, PointDipoleSource


def _source_fingerprint(objects: ObjectContainer, arrays: ArrayContainer) -> tuple:
    """Material values the source tables depend on (sources sample materials at setup)."""
    parts = []
    for s in objects.sources:
        sl = (slice(None), *s.grid_slice)
        if isinstance(s, (PointDipoleSource, LinearlyPolarizedPlaneSource)):
            parts.append(arrays.inv_permittivities[sl].detach().float().cpu().numpy().tobytes())
            mu = arrays.inv_permeabilities
            if isinstance(mu, torch.Tensor):
                parts.append(mu[sl].detach().float().cpu().numpy().tobytes())
    return tuple(parts)


def get_scene(objects: ObjectContainer, arrays: ArrayContainer, config: SimulationConfig,
              record_interfaces: bool = False) -> Scene:
    """The cached native scene of (objects, config, array layout); rebuilt when source inputs change."""
    cache = objects.__dict__.setdefault("_gb300_scenes", {})
    mu = arrays.inv_permeabilities
    key = (
        id(config), config.time, config.grid.spacing, config.courant_factor,
        tuple(arrays.inv_permittivities.shape),
        tuple(mu.shape) if isinstance(mu, torch.Tensor) else float(mu),
        None if arrays.electric_conductivity is None else tuple(arrays.electric_conductivity.shape),
        None if arrays.magnetic_conductivity is None else tuple(arrays.magnetic_conductivity.shape),
        None if arrays.dispersive_c1 is None else tuple(arrays.dispersive_c1.shape),
        record_interfaces,
    )
    fp = _source_fingerprint(objects, arrays)
    hit = cache.get(key)
    if hit is not None and hit[0] == fp:
        return hit[1]
    if hit is not None:
        hit[1].close()
    scene = Scene(objects, arrays, config, record_interfaces=record_interfaces)
    cache[key] = (fp, scene)
    return scene


def finite_status(scene: Scene) -> None:
    """Reads the plan's error word after a run that ended with a finite check.  A NaN or an
    infinity in the fields is reported with a ``RuntimeWarning`` and the arrays are still
    returned, as the reference returns a diverged run's arrays; any other error raises."""
    from fdtdx_gb300 import _native as N

    try:
        scene.status()
    except N.NativeError as e:
        if e.code != N.ENONFINITE:
            raise
        warnings.warn(f"the FDTD run diverged: {e}", RuntimeWarning, stacklevel=3)


def _materials_detached(arrays: ArrayContainer) -> ArrayContainer:
    mu = arrays.inv_permeabilities
    return arrays.aset("inv_permittivities", arrays.inv_permittivities.detach().contiguous()).aset(
        "inv_permeabilities", mu.detach().contiguous() if isinstance(mu, torch.Tensor) else mu
    )


def checkpointed_fdtd(
    arrays: ArrayContainer,
    objects: ObjectContainer,
    config: SimulationConfig,
    key=None,
    stopping_condition=None,
    show_progress: bool = True,
    progress_callback: Callable[[int, int], None] | None = None,
) -> SimulationState:
    """Forward run of ``config.time_steps_total`` steps from a reset state (fdtd.py:421-496)."""
    del key, show_progress
    if stopping_condition is not None:
        raise NotImplementedError("custom stopping conditions are not supported")
    if arrays.inv_permittivities.requires_grad and torch.is_grad_enabled():
        # the exact gradient through stored states (fdtd.py:421-496 differentiated by JAX)
        from fdtdx_gb300.adjoint import checkpointed_gradient_run

        out = checkpointed_gradient_run(arrays, objects, config)
        if progress_callback is not None:
            progress_callback(config.time_steps_total, config.time_steps_total)
        return config.time_steps_total, out
    arrays = _materials_detached(arrays).reset()
    scene = get_scene(objects, arrays, config, record_interfaces=config.invertible_optimization)
    T = config.time_steps_total
    scene.forward(arrays, 0, T, check_finite=True)
    finite_status(scene)
    if progress_callback is not None:
        progress_callback(T, T)
    return T, arrays


def run_fdtd(
    arrays: ArrayContainer,
    objects: ObjectContainer,
    config: SimulationConfig,
    key=None,
    stopping_condition=None,
    show_progress: bool = True,
    progress_callback: Callable[[int, int], None] | None = None,
) -> SimulationState:
    """Run the simulation; dispatches like fdtdx/fdtd/wrapper.py:14-63."""
    if stopping_condition is not None and config.gradient_config is not None:
        raise NotImplementedError(
            "Custom stopping conditions are not yet compatible with gradient computation."
        )
    gc = config.gradient_config
    if gc is None or gc.method == "checkpointed":
        return checkpointed_fdtd(arrays, objects, config, key, stopping_condition, show_progress, progress_callback)
    if gc.method == "reversible":
        from fdtdx_gb300.adjoint import reversible_fdtd

        return reversible_fdtd(arrays, objects, config, key, show_progress, progress_callback)
    raise Exception(f"Unknown gradient computation method: {gc.method}")
