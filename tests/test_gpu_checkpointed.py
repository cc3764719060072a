"""The exact checkpointed gradient (GradientConfig(method="checkpointed")) on the GPU.

The reference differentiates its checkpointed while loop with JAX (fdtdx/fdtd/fdtd.py:421-496);
here the forward run stores the state at the start of each of ``num_checkpoints`` segments and
the backward pass recomputes each segment's states and runs the transposed steps over them
(``fdtd_adjoint_stored``), with no time reversal.  So the gradient is exact everywhere, the
CPML included, and is checked against float64 autograd through the oracle's forward run over
the whole grid (relative L2 <= 1e-3), and against the reversible gradient in the interior
(the reference's own reversible-vs-checkpointed check, tests/simulation/fdtd/test_fdtd.py:394-463).
"""

from __future__ import annotations

import math

import pytest
import torch

import fdtdx_gb300 as fx
from oracle import fdtd_oracle as O
from tests.helpers import log_result, rel_l2
from tests.test_gpu_adjoint import _all_detectors_scene, _inner, _periodic_lossy_slab, _to_cuda

pytestmark = pytest.mark.gpu
GTOL = 1e-3


def _with_method(cfg, method, **kw):
    gc = fx.GradientConfig(method=method, recorder=fx.Recorder() if method == "reversible" else None, **kw)
    return fx.SimulationConfig(time=cfg.time, grid=cfg.grid, gradient_config=gc)


def _oracle_grad(objects, arrays, cfg, cE, cH, cots, dtype=torch.float64):
    """d <cot, outputs> / d inv_eps by autograd through the oracle's whole forward run."""
    sc = O.OracleScene(objects, arrays, cfg, dtype)
    ie = sc.inv_eps.clone().requires_grad_(True)
    st = sc.init_state()
    for _ in range(cfg.time_steps_total):
        st = O.forward(sc, st, inv_eps=ie)
    loss = _inner(cE.to(st.E.dtype), st.E) + _inner(cH.to(st.H.dtype), st.H)
    for (dn, k), c in cots.items():
        v = st.det[dn][k]
        loss = loss + _inner(c.to(v.dtype), v)
    (g,) = torch.autograd.grad(loss, [ie])
    return g


@pytest.mark.parametrize("segments", [1, 3])
def test_checkpointed_gradient_is_exact_with_cpml(segments):
    """Every detector kind, anisotropic lossy material, kappa != 1 CPML, plane and magnetic
    sources, seeded cotangents on E, H and every detector state: the checkpointed gradient
    against float64 autograd through the oracle over the whole grid (CPML cells included)."""
    objects, arrays, cfg0 = _all_detectors_scene(steps=40)
    cfg = _with_method(cfg0, "checkpointed", num_checkpoints=segments)
    g = torch.Generator().manual_seed(17)
    cots = {}
    for dn, st in arrays.detector_states.items():
        for k, v in st.items():
            cots[(dn, k)] = (torch.complex(torch.randn(v.shape, generator=g), torch.randn(v.shape, generator=g))
                             if v.is_complex() else torch.randn(v.shape, generator=g))
    cE = torch.randn(arrays.fields.E.shape, generator=g)
    cH = torch.randn(arrays.fields.H.shape, generator=g)
    ga = _to_cuda(objects, arrays)
    ie = ga.inv_permittivities.clone().requires_grad_(True)
    _, out = fx.run_fdtd(ga.aset("inv_permittivities", ie), objects, cfg)
    loss = _inner(cE.cuda(), out.fields.E) + _inner(cH.cuda(), out.fields.H)
    for (dn, k), c in cots.items():
        v = out.detector_states[dn][k]
        loss = loss + _inner(c.cuda().to(v.dtype), v)
    loss.backward()
    g_gpu = ie.grad.detach().cpu()
    g64 = _oracle_grad(objects, arrays, cfg, cE, cH, cots)
    e = rel_l2(g_gpu, g64)
    log_result(f"checkpointed_gradient_{segments}", grad_rel_l2_vs_fp64_autograd=e)
    assert torch.linalg.vector_norm(g64).item() > 0 and e <= GTOL, e


def test_checkpointed_and_reversible_gradients_agree():
    """The reference's scene for this check (a periodic lossy slab, loss sum(E^2) at the end):
    reversible and checkpointed gradients agree (no CPML, so the reversal is exact up to
    rounding)."""
    objects, arrays, cfg0 = _periodic_lossy_slab()
    grads = {}
    for method in ("reversible", "checkpointed"):
        cfg = _with_method(cfg0, method, **({"num_checkpoints": 4} if method == "checkpointed" else {}))
        ga = _to_cuda(objects, arrays)
        ie = ga.inv_permittivities.clone().requires_grad_(True)
        _, out = fx.run_fdtd(ga.aset("inv_permittivities", ie), objects, cfg)
        (out.fields.E ** 2).sum().backward()
        grads[method] = ie.grad.detach().cpu()
    e = rel_l2(grads["checkpointed"], grads["reversible"])
    log_result("checkpointed_vs_reversible", rel_l2=e)
    assert torch.linalg.vector_norm(grads["reversible"]).item() > 0 and e <= GTOL, e


def test_checkpointed_gradient_refusals():
    """Not provided, refused before any device work: the inv_permeabilities gradient and the
    gradient of dispersive materials."""
    objects, arrays, cfg0 = _periodic_lossy_slab()
    cfg = _with_method(cfg0, "checkpointed", num_checkpoints=2)
    ga = _to_cuda(objects, arrays)
    mu = torch.ones((1, *ga.inv_permittivities.shape[1:]), device="cuda", requires_grad=True)
    ie = ga.inv_permittivities.clone().requires_grad_(True)
    with pytest.raises(NotImplementedError):
        fx.run_fdtd(ga.aset("inv_permittivities", ie).aset("inv_permeabilities", mu), objects, cfg)
