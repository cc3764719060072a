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
  O(FdtdDesc, bloch_axes) O(FdtdDesc, bloch_sin) O(FdtdDesc, n_poles) O(FdtdDesc, n_disp)
  O(FdtdSourceDesc, e_table) O(FdtdSourceDesc, n_e_table)
  O(FdtdBuffers, psi_E) O(FdtdBuffers, det_state) O(FdtdBuffers, recording) O(FdtdBuffers, disp_P_curr)
  O(FdtdBuffers, disp_c3)
  O(FdtdAdjointBuffers, lam_det) O(FdtdAdjointBuffers, grad_inv_eps) O(FdtdAdjointBuffers, grad_inv_mu)
  O(FdtdAdjointBuffers, lam_P_prev)
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


def _valid_desc(nx=8, ny=8, nz=8):
    d = N.Desc()
    d.nx, d.ny, d.nz = nx, ny, nz
    d.n_steps_total = 4
    d.courant = 0.99 / 3**0.5
    d.n_eps = 1
    d.inv_mu_scalar = 1.0
    return d


@pytest.mark.parametrize("what", ["dims", "slab", "too_many_sources", "detector_box", "dipole_axis", "rec_dtype"])
def test_bad_descriptors_are_rejected_before_any_device_work(lib, what):
    """fdtd_plan_create validates the description on the host: an invalid one returns
    FDTD_EINVAL and no plan, before any CUDA call (so this runs without a GPU)."""
    import numpy as np

    d = _valid_desc()
    keep = []
    if what == "dims":
        d.nz = 0
    elif what == "slab":
        coef = np.zeros(6 * 20, np.float32)
        keep.append(coef)
        d.n_slabs = 1
        d.slabs[0].axis, d.slabs[0].direction, d.slabs[0].thickness = 0, -1, 20  # thicker than nx
        d.slabs[0].coef = coef.ctypes.data
    elif what == "too_many_sources":
        d.n_sources = N.MAX_SOURCES + 1
    elif what == "detector_box":
        slot = np.zeros(6, np.int32)
        keep.append(slot)
        d.n_detectors = 1
        dd = d.detectors[0]
        dd.kind, dd.comp_mask, dd.slot = N.DET_FIELD, 4, slot.ctypes.data
        for a in range(3):
            dd.lo[a], dd.hi[a] = 0, 8
        dd.hi[2] = 9  # one cell past the grid
    elif what == "dipole_axis":
        tab = np.zeros(6, np.float32)
        on = np.ones(6, np.uint8)
        keep += [tab, on]
        d.n_sources = 1
        so = d.sources[0]
        so.kind, so.component = N.SRC_DIPOLE, 3
        for a in range(3):
            so.lo[a], so.hi[a] = 4, 5
        so.phase_E = so.phase_H = so.teff = tab.ctypes.data
        so.on = on.ctypes.data
    elif what == "rec_dtype":
        d.recording_dtype = 7
    h = C.c_void_p(12345)
    rc = lib.fdtd_plan_create(C.byref(d), C.byref(h))
    assert rc == N.EINVAL and h.value is None


def test_debug_inject_rejects_unknown_kinds(lib):
    assert lib.fdtd_debug_inject(99, 1) == N.EINVAL
    assert lib.fdtd_debug_inject(N.INJECT_ALLOC, -1) == N.EINVAL
    assert lib.fdtd_debug_inject(N.INJECT_ALLOC, 0) == N.OK
    assert lib.fdtd_debug_inject(N.INJECT_WAIT_EXPIRY, 0) == N.OK
    assert lib.fdtd_debug_inject(N.INJECT_BARRIER_EXPIRY, 0) == N.OK
