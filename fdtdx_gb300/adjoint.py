"""Reversible (time-reversal) gradient: ``reversible_fdtd`` (fdtdx/fdtd/fdtd.py:39-418).

The forward pass runs on the native library and records the PML-interface planes
(``record_boundaries=config.invertible_optimization``).  The backward pass is the
reference's custom VJP: for t = T-1 down to -1, reconstruct the state at t by a
reverse step (interfaces re-imposed, psi frozen) and apply the transpose of the
forward step at t, accumulating d/d inv_permittivities and d/d inv_permeabilities
(the latter when the permeability is an array).  Both run in one native call
(``fdtd_adjoint``); here the cotangents are marshalled and the call is wrapped as a
``torch.autograd.Function``, the PyTorch counterpart of ``jax.custom_vjp``.

The sliced backward pass of ``num_checkpoints_reversible`` (fdtd.py:96-121, 292-322)
stores the full field state at the interior slice boundaries during the forward run
and resets the reconstruction to it when the backward loop reaches that step.

As in the reference only the materials receive a gradient (fdtd.py:324-333); the
initial fields, psi, detector states and recording get none.  A scalar (float)
inv_permeabilities carries no gradient here: make it a (1 | 3, nx, ny, nz) tensor to
differentiate it.
"""

from __future__ import annotations

from typing import Callable

import torch

from fdtdx_gb300.config import SimulationConfig
from fdtdx_gb300.container import ArrayContainer, FieldState, ObjectContainer, SimulationState


def reversible_slice_boundaries(time_steps_total: int, num_slices: int) -> list[int]:
    """Slice boundaries [s_0 = 0, ..., s_k = T] of the sliced backward pass (fdtd.py:20-36)."""
    return [round(i * time_steps_total / num_slices) for i in range(num_slices + 1)]


def _clone_fields(f: FieldState) -> FieldState:
    return FieldState(
        E=f.E.clone(),
        H=f.H.clone(),
        psi_E={k: (a.clone(), b.clone()) for k, (a, b) in f.psi_E.items()},
        psi_H={k: (a.clone(), b.clone()) for k, (a, b) in f.psi_H.items()},
        dispersive_P_curr=None if f.dispersive_P_curr is None else f.dispersive_P_curr.clone(),
        dispersive_P_prev=None if f.dispersive_P_prev is None else f.dispersive_P_prev.clone(),
    )


def _copy_fields(dst: FieldState, src: FieldState) -> None:
    dst.E.copy_(src.E)
    dst.H.copy_(src.H)
    for k in dst.psi_E:
        dst.psi_E[k][0].copy_(src.psi_E[k][0])
        dst.psi_E[k][1].copy_(src.psi_E[k][1])
        dst.psi_H[k][0].copy_(src.psi_H[k][0])
        dst.psi_H[k][1].copy_(src.psi_H[k][1])
    if dst.dispersive_P_curr is not None:
        dst.dispersive_P_curr.copy_(src.dispersive_P_curr)
        dst.dispersive_P_prev.copy_(src.dispersive_P_prev)


class _Layout:
    """Flat tensor order of the run's outputs: E, H, psi_E, psi_H, detector states."""

    def __init__(self, arrays: ArrayContainer):
        f = arrays.fields
        self.pml_names = list(f.psi_E.keys())
        self.det_keys = [(n, k) for n, st in arrays.detector_states.items() for k in st]

    def flatten(self, arrays: ArrayContainer) -> list[torch.Tensor]:
        f = arrays.fields
        out = [f.E, f.H]
        for n in self.pml_names:
            out += [f.psi_E[n][0], f.psi_E[n][1]]
        for n in self.pml_names:
            out += [f.psi_H[n][0], f.psi_H[n][1]]
        out += [arrays.detector_states[n][k] for n, k in self.det_keys]
        return out

    def unflatten(self, arrays: ArrayContainer, flat: list[torch.Tensor]) -> ArrayContainer:
        it = iter(flat)
        E, H = next(it), next(it)
        psi_E = {n: (next(it), next(it)) for n in self.pml_names}
        psi_H = {n: (next(it), next(it)) for n in self.pml_names}
        det: dict[str, dict[str, torch.Tensor]] = {n: {} for n in arrays.detector_states}
        for n, k in self.det_keys:
            det[n][k] = next(it)
        arrays = arrays.aset("fields", FieldState(E=E, H=H, psi_E=psi_E, psi_H=psi_H))
        return arrays.aset("detector_states", det)


class _ReversibleRun(torch.autograd.Function):
    """Forward run + reversible backward; the differentiable inputs are the materials."""

    @staticmethod
    def forward(ctx, ctl: dict, inv_eps: torch.Tensor, inv_mu: torch.Tensor | None):
        scene, arrays, T = ctl["scene"], ctl["arrays"], ctl["T"]
        bounds = ctl["bounds"]
        checkpoints = []
        for seg in range(len(bounds) - 1):
            scene.forward(arrays, bounds[seg], bounds[seg + 1] - bounds[seg], check_finite=seg == len(bounds) - 2)
            if seg < len(bounds) - 2:
                checkpoints.append(_clone_fields(arrays.fields))
        from fdtdx_gb300.fdtd import finite_status

        finite_status(scene)
        ctl["checkpoints"] = checkpoints
        ctl["final"] = arrays
        ctx.ctl = ctl
        # the outputs are aliases of the final state: autograd attaches its node to the aliases,
        # so the state held by the node's context does not point back at the node (no cycle)
        return tuple(t.detach() for t in ctl["layout"].flatten(arrays))

    @staticmethod
    def backward(ctx, *grads):
        ctl = ctx.ctl
        scene, layout, T = ctl["scene"], ctl["layout"], ctl["T"]
        final: ArrayContainer = ctl["final"]
        bounds, checkpoints = ctl["bounds"], ctl["checkpoints"]
        # reconstruct on a copy: the outputs handed to the caller stay intact
        state = final.aset("fields", _clone_fields(final.fields))
        f = state.fields
        outs = layout.flatten(final)

        def cot(i):
            g = grads[i]
            if g is None:
                return torch.zeros_like(outs[i])
            return g.detach().to(outs[i].dtype).contiguous().clone()

        lam = {"E": cot(0), "H": cot(1)}
        i = 2
        lam["psi_E"] = {}
        for n in layout.pml_names:
            lam["psi_E"][n] = (cot(i), cot(i + 1))
            i += 2
        lam["psi_H"] = {}
        for n in layout.pml_names:
            lam["psi_H"][n] = (cot(i), cot(i + 1))
            i += 2
        lam["det"] = {}
        for n, _k in layout.det_keys:
            if grads[i] is not None:
                lam["det"][n] = cot(i)
            i += 1
        ie, im = ctl["inv_eps"], ctl["inv_mu"]
        want_eps, want_mu = ctx.needs_input_grad[1], ctx.needs_input_grad[2]
        grad = grad_mu = None
        if want_eps:
            grad = torch.zeros_like(ie, dtype=torch.float32).contiguous()
            lam["grad_inv_eps"] = grad
        if want_mu:
            grad_mu = torch.zeros_like(im, dtype=torch.float32).contiguous()
            lam["grad_inv_mu"] = grad_mu
        # slices from the last to the first; the last call runs down to t = -1
        k = len(bounds) - 1
        for seg in range(k - 1, -1, -1):
            t_end = bounds[seg + 1]
            n = t_end - bounds[seg] + (1 if seg == 0 else 0)
            scene.adjoint(state, lam, t_end, n)
            if seg > 0:
                _copy_fields(f, checkpoints[seg - 1])
        scene.status()
        ctl["checkpoints"] = []
        return (None, None if grad is None else grad.to(ie.dtype),
                None if grad_mu is None else grad_mu.to(im.dtype))


def reversible_fdtd(
    arrays: ArrayContainer,
    objects: ObjectContainer,
    config: SimulationConfig,
    key=None,
    show_progress: bool = True,
    progress_callback: Callable[[int, int], None] | None = None,
) -> SimulationState:
    """Differentiable forward run with the time-reversal gradient (fdtd.py:39-418).

    Returns ``(T, arrays)`` like the reference.  When ``arrays.inv_permittivities`` or an
    array ``arrays.inv_permeabilities`` requires a gradient, the returned fields and
    detector states are connected to it through the reversible backward pass.
    """
    del key, show_progress
    from fdtdx_gb300.fdtd import _materials_detached, get_scene

    if arrays.dispersive_c1 is not None or arrays.fields.dispersive_P_curr is not None:
        # as the reference (fdtd.py:98-104): the ADE polarisation cannot be time-reversed
        raise NotImplementedError("reversible_fdtd does not support dispersive materials: use the checkpointed "
                                  "gradient method for dispersive simulations")

    gc = config.gradient_config
    num_ckpt = 0 if gc is None else gc.num_checkpoints_reversible
    T = config.time_steps_total
    num_slices = num_ckpt + 1
    if num_ckpt > 0 and num_slices > T:
        raise Exception(
            "num_checkpoints_reversible must be <= time_steps_total - 1 "
            f"(got num_checkpoints_reversible={num_ckpt}, time_steps_total={T})"
        )
    bounds = reversible_slice_boundaries(T, num_slices)
    ie_in = arrays.inv_permittivities
    mu_in = arrays.inv_permeabilities
    if isinstance(mu_in, torch.Tensor) and mu_in.dim() == 0:
        if mu_in.requires_grad:
            raise NotImplementedError("a 0-d inv_permeabilities has no gradient here: pass a (1|3, nx, ny, nz) array")
        mu_in = float(mu_in)
        arrays = arrays.aset("inv_permeabilities", mu_in)
    mu_t = mu_in if isinstance(mu_in, torch.Tensor) else None
    work = _materials_detached(arrays).reset()
    if work.recording_state is None and config.invertible_optimization and objects.pml_objects:
        raise ValueError("the reversible gradient needs a recording state (init_arrays with a recorder)")
    scene = get_scene(objects, work, config, record_interfaces=config.invertible_optimization)
    layout = _Layout(work)
    ctl = {"scene": scene, "arrays": work, "T": T, "bounds": bounds, "layout": layout,
           "inv_eps": work.inv_permittivities, "inv_mu": work.inv_permeabilities}
    wants = ie_in.requires_grad or (mu_t is not None and mu_t.requires_grad)
    if wants and torch.is_grad_enabled() and scene.full_tensor:
        raise NotImplementedError("the reversible gradient of full 3x3 tensor materials is not supported by the GB300 "
                                  "kernels (their forward and reverse steps are)")
    if wants and torch.is_grad_enabled() and scene.complex_fields and mu_t is not None and mu_t.requires_grad:
        raise NotImplementedError("the inv_permeabilities gradient of complex (Bloch) fields is not supported by the "
                                  "GB300 kernels (the inv_permittivities gradient is)")
    if not (torch.is_grad_enabled() and wants):
        _ReversibleRun.forward(_NoCtx(), ctl, work.inv_permittivities, None)
        out = work
    else:
        flat = _ReversibleRun.apply(ctl, ie_in, mu_t)
        out = layout.unflatten(work, list(flat))
        out = out.aset("inv_permittivities", ie_in)
        if mu_t is not None:
            out = out.aset("inv_permeabilities", mu_t)
    if progress_callback is not None:
        progress_callback(T, T)
    return T, out


class _NoCtx:
    """Stand-in context for a forward run that needs no backward."""


class _CheckpointedRun(torch.autograd.Function):
    """The exact gradient of GradientConfig(method="checkpointed") (the reference differentiates
    its checkpointed while loop, fdtdx/fdtd/fdtd.py:421-496): the forward run stores the full
    state (the dispersive polarisation included) at the start of each of ``num_checkpoints``
    segments; the backward pass, from the last segment to the first, recomputes the segment's
    states from its checkpoint and runs the transposed steps over them
    (``fdtd_adjoint_stored``, the ADE step transposed too).  No reconstruction is involved, so
    the gradient is exact everywhere, inside the CPML included.  Memory: the checkpoints plus
    one segment of states."""

    @staticmethod
    def forward(ctx, ctl: dict, inv_eps: torch.Tensor, inv_mu):
        scene, arrays, bounds = ctl["scene"], ctl["arrays"], ctl["bounds"]
        checkpoints = []
        for seg in range(len(bounds) - 1):
            checkpoints.append(_clone_fields(arrays.fields))
            scene.forward(arrays, bounds[seg], bounds[seg + 1] - bounds[seg], check_finite=seg == len(bounds) - 2)
        from fdtdx_gb300.fdtd import finite_status

        finite_status(scene)
        ctl["checkpoints"] = checkpoints
        ctl["final"] = arrays
        ctx.ctl = ctl
        return tuple(t.detach() for t in ctl["layout"].flatten(arrays))

    @staticmethod
    def backward(ctx, *grads):
        ctl = ctx.ctl
        scene, layout, bounds = ctl["scene"], ctl["layout"], ctl["bounds"]
        final: ArrayContainer = ctl["final"]
        outs = layout.flatten(final)

        def cot(i):
            g = grads[i]
            if g is None:
                return torch.zeros_like(outs[i])
            return g.detach().to(outs[i].dtype).contiguous().clone()

        lam = {"E": cot(0), "H": cot(1)}
        i = 2
        lam["psi_E"], lam["psi_H"] = {}, {}
        for n in layout.pml_names:
            lam["psi_E"][n] = (cot(i), cot(i + 1))
            i += 2
        for n in layout.pml_names:
            lam["psi_H"][n] = (cot(i), cot(i + 1))
            i += 2
        lam["det"] = {}
        for n, _k in layout.det_keys:
            if grads[i] is not None:
                lam["det"][n] = cot(i)
            i += 1
        ie = ctl["inv_eps"]
        grad = torch.zeros_like(ie, dtype=torch.float32).contiguous()
        lam["grad_inv_eps"] = grad
        if final.fields.dispersive_P_curr is not None:  # the polarisation is no output: zero cotangents
            lam["P_curr"] = torch.zeros_like(final.fields.dispersive_P_curr)
            lam["P_prev"] = torch.zeros_like(final.fields.dispersive_P_prev)
        # recompute on scratch state (the detector states accumulate there and are discarded)
        work = final.aset("fields", _clone_fields(final.fields)).aset(
            "detector_states", {k: {k2: v2.clone() for k2, v2 in v.items()} for k, v in final.detector_states.items()})
        for seg in range(len(bounds) - 2, -1, -1):
            t0, L = bounds[seg], bounds[seg + 1] - bounds[seg]
            _copy_fields(work.fields, ctl["checkpoints"][seg])
            states = [_clone_fields(work.fields)]
            for q in range(L):
                scene.forward(work, t0 + q, 1, graph=False)
                states.append(_clone_fields(work.fields))
            scene.adjoint_stored(work, states, t0, lam)
            del states
        scene.status()
        return None, grad.to(ie.dtype), None


def checkpointed_gradient_run(arrays: ArrayContainer, objects: ObjectContainer, config: SimulationConfig):
    """The forward run of checkpointed_fdtd connected to d/d inv_permittivities through the
    exact stored-state backward pass (``_CheckpointedRun``); returns the output container."""
    from fdtdx_gb300.fdtd import _materials_detached, get_scene

    gc = config.gradient_config
    if gc is None or gc.num_checkpoints is None:
        raise Exception("Need Checkpoint Number in gradient config to compute checkpointed gradients")
    mu = arrays.inv_permeabilities
    if isinstance(mu, torch.Tensor) and mu.requires_grad:
        raise NotImplementedError("the checkpointed gradient provides d/d inv_permittivities only")
    T = config.time_steps_total
    n_seg = max(1, min(int(gc.num_checkpoints), T))
    bounds = reversible_slice_boundaries(T, n_seg)
    ie_in = arrays.inv_permittivities
    work = _materials_detached(arrays).reset()
    scene = get_scene(objects, work, config, record_interfaces=False)
    if scene.complex_fields or scene.full_tensor:
        raise NotImplementedError("the checkpointed gradient of complex (Bloch) fields or full 3x3 tensor materials "
                                  "is not supported by the GB300 kernels")
    layout = _Layout(work)
    ctl = {"scene": scene, "arrays": work, "bounds": bounds, "layout": layout, "inv_eps": work.inv_permittivities}
    flat = _CheckpointedRun.apply(ctl, ie_in, None)
    out = layout.unflatten(work, list(flat))
    return out.aset("inv_permittivities", ie_in)
