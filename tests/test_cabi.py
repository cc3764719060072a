"""The C-ABI library loads, exports every symbol the header declares, and the ctypes
mirrors have the C compiler's layout.  No compute calls (no GPU needed)."""

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from fdtdx_gb300 import _native as N
from fdtdx_gb300.build import build

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "fdtd_gb300.h"


def declared_functions() -> set[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(fdtd_[a-z0-9_]+)\s*\(", text))


@pytest.fixture(scope="module")
def lib():
    build()
    return N.load()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert names, "no declarations parsed"
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert names == set(N.SIGNATURES), "ctypes signatures and header declarations differ"
    out = subprocess.run(["nm", "-D", "--defined-only", str(N.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fdtd_[a-z0-9_]+)", out))
    assert names <= exported


_PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "fdtd_gb300.h"
#define P(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  P(FdtdSlabDesc) P(FdtdSourceDesc) P(FdtdDetectorDesc) P(FdtdDesc) P(FdtdBuffers) P(FdtdAdjointBuffers)
  O(FdtdSourceDesc, inc_E) O(FdtdSourceDesc, profile) O(FdtdSourceDesc, phase_E) O(FdtdSourceDesc, on)
  O(FdtdDetectorDesc, cell_weight) O(FdtdDetectorDesc, slot) O(FdtdDetectorDesc, weights)
  O(FdtdDesc, slabs) O(FdtdDesc, n_sources) O(FdtdDesc, sources) O(FdtdDesc, detectors) O(FdtdDesc, recording_dtype)
  O(FdtdBuffers, psi_E) O(FdtdBuffers, det_state) O(FdtdBuffers, recording)
  O(FdtdAdjointBuffers, lam_det) O(FdtdAdjointBuffers, grad_inv_eps) O(FdtdAdjointBuffers, grad_inv_mu)
  return 0;
}
"""


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(_PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(HEADER.parent), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")
               if line)
    m = {"FdtdSlabDesc": N.SlabDesc, "FdtdSourceDesc": N.SourceDesc, "FdtdDetectorDesc": N.DetectorDesc,
         "FdtdDesc": N.Desc, "FdtdBuffers": N.Buffers, "FdtdAdjointBuffers": N.AdjointBuffers}
    for key, val in got.items():
        if "." in key:
            t, f = key.split(".")
            assert getattr(m[t], f).offset == int(val), key
        else:
            assert C.sizeof(m[key]) == int(val), key
