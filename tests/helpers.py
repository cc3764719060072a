"""Shared helpers of the parity tests."""

from __future__ import annotations

import json
import os
import tempfile
from pathlib import Path

import torch

from oracle import fdtd_oracle as O

# parity records (measured errors per case); FDTD_PARITY_LOG chooses the file
RESULTS = Path(os.environ.get("FDTD_PARITY_LOG", os.path.join(tempfile.gettempdir(), "fdtd_parity.jsonl")))


def rel_l2(a, b) -> float:
    a = torch.as_tensor(a).detach().cpu().to(torch.complex128 if torch.as_tensor(a).is_complex() else torch.float64)
    b = torch.as_tensor(b).detach().cpu().to(a.dtype)
    nb = torch.linalg.vector_norm(b).item()
    d = torch.linalg.vector_norm(a - b).item()
    return d / nb if nb > 0 else d


def log_result(name: str, **kw) -> None:
    """Append a parity record (read when the tolerance table of the design notes is updated)."""
    try:
        RESULTS.parent.mkdir(parents=True, exist_ok=True)
        with RESULTS.open("a") as f:
            f.write(json.dumps({"case": name, **kw}) + "\n")
    except OSError:
        pass


def oracle_run(objects, arrays, config, dtype, steps=None, state=None, record=False):
    sc = O.OracleScene(objects, arrays, config, dtype=dtype)
    st = O.run(sc, steps, record_boundaries=record, state=state)
    return sc, st


def compare_states(name, arrays, ref32, ref64, tol=1e-4, keys=None) -> dict:
    """rel L2 of fields and detector states vs the float32 (asserted) and float64 (reported) oracles."""
    out = {}
    pairs = {"E": (arrays.fields.E, ref32.E, ref64.E), "H": (arrays.fields.H, ref32.H, ref64.H)}
    for dn, st in arrays.detector_states.items():
        for k, v in st.items():
            pairs[f"{dn}.{k}"] = (v, ref32.det[dn][k], ref64.det[dn][k])
    for k, (g, r32, r64) in pairs.items():
        if keys is not None and k not in keys:
            continue
        e32, e64 = rel_l2(g, r32), rel_l2(g, r64)
        out[k] = {"rel_l2_vs_fp32": e32, "rel_l2_vs_fp64": e64, "fp32_oracle_vs_fp64": rel_l2(r32, r64)}
    log_result(name, **out)
    for k, v in out.items():
        assert v["rel_l2_vs_fp32"] <= tol, (name, k, v)
    return out
