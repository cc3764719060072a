"""The serving loop: every result in the mix equals the same job run alone.

Six requests (forward and gradient, isotropic and diagonal-anisotropic, uneven grids and
step counts) arrive staggered on a virtual clock, with a budget that holds only part of
them at once, so jobs queue, join a running batch, leave it, and gradient jobs run their
adjoint phase while others are still in their forward phase.  Tolerance: relative L2
<= 1e-5 on fields, detector states, losses and gradients against the alone run (the
batch runs the register-queue core where a single run may use the TMA core).
"""

import pytest
import torch

from fdtdx_gb300.serving import Server, estimate_footprint, latency_stats, random_boxes_job, run_one_at_a_time
from tests.helpers import log_result, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _jobs():
    specs = [
        ((40, 36, 32), 160, 1, "forward", False, 0.0),
        ((32, 44, 36), 120, 2, "gradient", False, 0.0),
        ((48, 40, 30), 200, 3, "forward", True, 0.001),
        ((36, 36, 36), 90, 4, "gradient", True, 0.002),
        ((30, 34, 33), 140, 5, "forward", False, 0.003),
        ((44, 32, 40), 110, 6, "forward", False, 0.004),
    ]
    return [random_boxes_job(s, steps=t, seed=seed, kind=kind, anisotropic=an, arrival=arr)
            for s, t, seed, kind, an, arr in specs]


def test_served_results_equal_alone_runs():
    mix = _jobs()
    fps = sorted(estimate_footprint(j) for j in mix)
    budget = sum(fps[-3:])  # about three jobs at once: the rest queue
    server = Server(budget_bytes=budget, max_slots=4, target_chunk_s=0.002)
    server.run(mix, realtime=False)
    alone = run_one_at_a_time(_jobs(), realtime=False)
    assert all(j.phase == "done" for j in mix)
    assert max(j.t_admit for j in mix) > 0.0  # something had to wait for memory
    for j, r in zip(sorted(mix, key=lambda x: x.id), sorted(alone, key=lambda x: x.id)):
        if j.kind == "gradient":
            e_g = rel_l2(j.grad, r.grad)
            e_l = abs(j.loss_value - r.loss_value) / abs(r.loss_value)
            e_d = max(rel_l2(v, r.detectors[n][k]) for n, s in j.detectors.items() for k, v in s.items())
            log_result(f"serving_gradient_{j.id}", grad=e_g, loss=e_l, detectors=e_d)
            assert torch.linalg.vector_norm(r.grad).item() > 0
            assert e_g <= TOL and e_l <= TOL and e_d <= TOL, (j.id, e_g, e_l, e_d)
        else:
            errs = {"E": rel_l2(j.result.fields.E, r.result.fields.E), "H": rel_l2(j.result.fields.H, r.result.fields.H)}
            for n, s in j.result.detector_states.items():
                for k, v in s.items():
                    errs[f"{n}.{k}"] = rel_l2(v, r.result.detector_states[n][k])
            log_result(f"serving_forward_{j.id}", **errs)
            for k, e in errs.items():
                assert e <= TOL, (j.id, k, e)
    st = latency_stats(mix)
    assert st["p50_s"] is not None and st["p99_s"] >= st["p50_s"]
