"""Recorder time filter (LinearReconstructEveryK, fdtdx/interfaces/time_filter.py:140-257).

Known answers from the reference's own tests (tests/unit/interfaces/test_time_filter.py:39-163):
the last step is always stored, the first stored step is start_recording_after, k = 1 keeps
every step, a stored step reads its slot, and the midpoint between two slots interpolates
to the midpoint.  The product's per-step tables must also agree with the oracle's
restatement at every step, t = -1 included.
"""

import types

import numpy as np
import pytest
import torch

from fdtdx_gb300.config import GradientConfig, LinearReconstructEveryK, Recorder
from oracle import fdtd_oracle as O


def test_known_answers():
    assert 49 in LinearReconstructEveryK(k=7).save_steps(50)
    assert LinearReconstructEveryK(k=10, start_recording_after=20).save_steps(100)[0] == 20
    assert len(LinearReconstructEveryK(k=1).save_steps(50)) == 50
    store, a, b, w = LinearReconstructEveryK(k=10).tables(100)
    assert store[0 + 1] == 0 and store[10 + 1] == 1 and store[5 + 1] == -1
    assert (a[5 + 1], b[5 + 1]) == (0, 1) and abs(w[5 + 1] - 0.5) < 1e-12  # 0 -> 10: value 5 at t = 5
    assert Recorder([LinearReconstructEveryK(k=4)]).slots(30) == len(range(0, 30, 4)) + 1


def _oracle_scene(T, k, start):
    sc = O.OracleScene.__new__(O.OracleScene)
    sc.T = T
    cfg = types.SimpleNamespace(gradient_config=GradientConfig(
        recorder=Recorder([LinearReconstructEveryK(k=k, start_recording_after=start)])))
    sc._setup_time_filter(cfg)
    return sc


@pytest.mark.parametrize("T,k,start", [(30, 4, 0), (37, 5, 3), (12, 1, 0), (50, 7, 10)])
def test_tables_match_oracle(T, k, start):
    tf = LinearReconstructEveryK(k=k, start_recording_after=start)
    store, ra, rb, rw = tf.tables(T)
    sc = _oracle_scene(T, k, start)
    slots = len(tf.save_steps(T))
    rec = [{"v": torch.tensor([float(3 * q + 1), float(-q)], dtype=torch.float64)} for q in range(slots)]
    for t in range(-1, T):
        assert (store[t + 1] >= 0) == sc.records(t), t
        want = sc.recorded(rec, t)["v"]
        va, vb = rec[ra[t + 1]]["v"], rec[rb[t + 1]]["v"]
        got = va + rw[t + 1] * (vb - va)
        assert torch.allclose(got, want, rtol=1e-12, atol=1e-12), (t, got, want)
    # the stored slots are exactly 0 .. slots-1, in step order
    stored = [s for s in store[1:T + 1] if s >= 0]
    assert stored == list(range(slots))
