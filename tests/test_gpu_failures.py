"""Failure detection on the GPU path, with no GPU fault involved.

* A bounded pipeline wait that runs out: ``fdtd_debug_inject(FDTD_INJECT_WAIT_EXPIRY)``
  makes a TMA half-step take its error exit before it issues any copy; the error word
  reaches ``fdtd_plan_status`` as FDTD_ETIMEOUT and ``Scene.status()`` raises.  The context
  stays usable: the next run equals an undisturbed one bit for bit.
* A failed device allocation: ``FDTD_INJECT_ALLOC`` makes the plan's (and the adjoint
  scratch's) allocation report out-of-memory: FDTD_ENOMEM, and the next build succeeds.
* A diverged run: a NaN planted in the permittivity on the host side makes the finite
  check report FDTD_ENONFINITE; ``run_fdtd`` warns and returns the arrays, as the reference
  returns a diverged run's arrays.
* The serving loop: a queued and a running job are cancelled, one job diverges; it fails
  alone, and every other job's result equals its run alone.
"""

from __future__ import annotations

import pytest
import torch

import fdtdx_gb300 as fx
from fdtdx_gb300 import _native as N
from fdtdx_gb300 import scenes
from fdtdx_gb300.engine import Scene
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _clear_injections():
    yield
    lib = N.load()
    lib.fdtd_debug_inject(N.INJECT_ALLOC, 0)
    lib.fdtd_debug_inject(N.INJECT_WAIT_EXPIRY, 0)


def _tma_scene():
    objects, arrays, _, cfg, _ = scenes.coupler(shape=(48, 44, 32), steps=40, scale=0.3, pml=6, device="cuda")
    return objects, arrays, cfg


def test_injected_wait_expiry_reaches_status_and_the_context_stays_usable():
    objects, arrays, cfg = _tma_scene()
    ref = arrays.reset()
    s = Scene(objects, ref, cfg)
    assert s.uses_tma
    s.forward(ref, 0, 20, graph=False)
    s.status()
    bad = arrays.reset()
    s.forward(bad, 0, 10, graph=False)
    assert N.load().fdtd_debug_inject(N.INJECT_WAIT_EXPIRY, 1) == N.OK
    s.forward(bad, 10, 10, graph=False)
    with pytest.raises(N.NativeError) as ei:
        s.status()
    assert ei.value.code == N.ETIMEOUT
    s.status()  # the word was read and cleared
    again = arrays.reset()
    s.forward(again, 0, 20, graph=False)
    s.status()
    torch.cuda.synchronize()
    assert torch.equal(again.fields.E, ref.fields.E) and torch.equal(again.fields.H, ref.fields.H)
    assert not torch.equal(bad.fields.E, ref.fields.E)  # the expired launch updated nothing
    s.close()


def test_injected_allocation_failure_is_enomem():
    objects, arrays, cfg = _tma_scene()
    lib = N.load()
    assert lib.fdtd_debug_inject(N.INJECT_ALLOC, 1) == N.OK
    s = Scene(objects, arrays.reset(), cfg)
    with pytest.raises(N.NativeError) as ei:
        s.plan
    assert ei.value.code == N.ENOMEM
    s2 = Scene(objects, arrays.reset(), cfg)  # the injection was consumed: this one builds
    assert s2.plan
    s2.close()


def test_injected_adjoint_scratch_failure_is_enomem():
    objects, arrays, _, cfg, _ = scenes.inverse_design(shape=(28, 28, 24), steps=30, design=(8, 8, 3), plane=(6, 6),
                                                       pml=5, device="cuda")
    ie = arrays.inv_permittivities.clone().requires_grad_(True)
    _, out = fx.reversible_fdtd(arrays.aset("inv_permittivities", ie), objects, cfg)
    loss = (out.detector_states["objective"]["phasor"].abs() ** 2).sum()
    assert N.load().fdtd_debug_inject(N.INJECT_ALLOC, 1) == N.OK
    with pytest.raises(N.NativeError) as ei:
        loss.backward()
    assert ei.value.code == N.ENOMEM


def test_nonfinite_field_is_detected():
    objects, arrays, _, cfg, _ = scenes.dipole_boxes(shape=(24, 24, 24), steps=30, n_boxes=3, pml=5, device="cuda")
    poisoned = arrays.aset("inv_permittivities", arrays.inv_permittivities.clone())
    poisoned.inv_permittivities[0, 9, 12, 12] = float("nan")
    with pytest.warns(RuntimeWarning, match="diverged"):
        _, out = fx.run_fdtd(poisoned, objects, cfg)
    assert not torch.isfinite(out.fields.E).all()
    s = Scene(objects, poisoned.reset(), cfg)
    w = poisoned.reset()
    s.forward(w, 0, 30, check_finite=True)
    with pytest.raises(N.NativeError) as ei:
        s.status()
    assert ei.value.code == N.ENONFINITE
    ok = arrays.reset()
    s2 = Scene(objects, ok, cfg)
    s2.forward(ok, 0, 30, check_finite=True)
    s2.status()  # a finite run reports nothing
    s.close()
    s2.close()


def test_serving_cancellation_and_divergence_are_isolated():
    from fdtdx_gb300.serving import Job, Server, random_boxes_job, run_one_at_a_time

    def poisoned_job(arrival):
        base = random_boxes_job((30, 32, 28), steps=120, seed=44, arrival=arrival)

        def build(device, with_recorder):
            o, a, c = base.build(device, with_recorder)
            a = a.aset("inv_permittivities", a.inv_permittivities.clone())
            a.inv_permittivities[0, 15, 16, 14] = float("nan")
            return o, a, c

        return Job(build=build, kind="forward", arrival=arrival)

    def mix():
        return [
            random_boxes_job((36, 32, 30), steps=200, seed=41, arrival=0.0),                      # 0 runs
            random_boxes_job((32, 36, 28), steps=160, seed=42, kind="gradient", arrival=0.0),      # 1 runs
            random_boxes_job((40, 36, 32), steps=400, seed=43, arrival=0.0),                      # 2 cancelled running
            poisoned_job(0.0),                                                                    # 3 diverges
            random_boxes_job((30, 30, 30), steps=150, seed=45, arrival=0.001),                    # 4 cancelled queued
        ]

    jobs = mix()
    server = Server(budget_bytes=10**12, max_slots=4, target_chunk_s=0.002)
    seen = {}

    def on_chunk(srv, now):
        if "snap" not in seen and jobs[2].phase == "forward" and jobs[2].t_fwd > 0:
            seen["snap"] = srv.snapshot(jobs[2])
            srv.cancel(jobs[2])
            srv.cancel(jobs[4])

    server.run(jobs, realtime=False, on_chunk=on_chunk)
    assert [j.phase for j in jobs] == ["done", "done", "cancelled", "failed", "cancelled"]
    assert "NaN" in jobs[3].error or "infinity" in jobs[3].error
    assert seen["snap"]["E"].shape == (3, 40, 36, 32) and 0 < seen["snap"]["t"] <= 400
    assert jobs[2].result is None and jobs[4].result is None
    assert server.sched.used == 0
    alone = run_one_at_a_time(mix()[:2], realtime=False)
    assert rel_l2(jobs[0].result.fields.E, alone[0].result.fields.E) <= 1e-5
    assert rel_l2(jobs[1].grad, alone[1].grad) <= 1e-5
