"""ctypes binding of ``libfdtd_gb300.so`` (declared in include/fdtd_gb300.h).

The structures below mirror the C structs field by field; ``tests/test_cabi.py``
checks their sizes and offsets against the C compiler's.  Loading fails loudly
when the library is missing: there is no CPU fallback of the time-stepping path.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

MAX_SLABS = 6
MAX_SOURCES = 16
MAX_DETECTORS = 32
MAX_FREQS = 16

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, ENONFINITE = range(6)
FWD_GRAPH, FWD_CHECK_FINITE = 1, 2
INJECT_ALLOC, INJECT_WAIT_EXPIRY, INJECT_BARRIER_EXPIRY = 1, 2, 3
PROFILE_CW, PROFILE_GAUSSIAN = 0, 1
SRC_DIPOLE, SRC_PLANE = 0, 1
DET_FIELD, DET_PHASOR, DET_FLUX, DET_ENERGY = 0, 1, 2, 3

_fp = C.POINTER(C.c_float)


class SlabDesc(C.Structure):
    _fields_ = [
        ("axis", C.c_int32),
        ("direction", C.c_int32),
        ("thickness", C.c_int32),
        ("kappa_is_one", C.c_int32),
        ("coef", C.c_void_p),
    ]


class SourceDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("lo", C.c_int32 * 3),
        ("hi", C.c_int32 * 3),
        ("component", C.c_int32),
        ("magnetic", C.c_int32),
        ("normal_axis", C.c_int32),
        ("sign", C.c_float),
        ("coef", C.c_float),
        ("inc_E", C.c_void_p),
        ("inc_H", C.c_void_p),
        ("off_E", C.c_void_p),
        ("off_H", C.c_void_p),
        ("profile", C.c_int32),
        ("omega_dt", C.c_float),
        ("ramp_inv_steps", C.c_float),
        ("t0_steps", C.c_float),
        ("inv_two_sigma2", C.c_float),
        ("phase_E", C.c_void_p),
        ("phase_H", C.c_void_p),
        ("teff", C.c_void_p),
        ("on", C.c_void_p),
        ("e_table", C.c_void_p),
        ("n_e_table", C.c_int32),
    ]


class DetectorDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("lo", C.c_int32 * 3),
        ("hi", C.c_int32 * 3),
        ("comp_mask", C.c_int32),
        ("exact_interpolation", C.c_int32),
        ("reduce_volume", C.c_int32),
        ("inverse", C.c_int32),
        ("n_freq", C.c_int32),
        ("flux_axis", C.c_int32),
        ("flux_sign", C.c_float),
        ("keep_all", C.c_int32),
        ("cell_weight", C.c_float),
        ("slot", C.c_void_p),
        ("weights", C.c_void_p),
    ]


class Desc(C.Structure):
    _fields_ = [
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nz", C.c_int32),
        ("n_steps_total", C.c_int32),
        ("courant", C.c_float),
        ("n_eps", C.c_int32),
        ("n_mu", C.c_int32),
        ("inv_mu_scalar", C.c_float),
        ("n_sigma_E", C.c_int32),
        ("n_sigma_H", C.c_int32),
        ("periodic", C.c_int32 * 3),
        ("pec_faces", C.c_int32),
        ("pmc_faces", C.c_int32),
        ("n_slabs", C.c_int32),
        ("slabs", SlabDesc * MAX_SLABS),
        ("n_sources", C.c_int32),
        ("sources", SourceDesc * MAX_SOURCES),
        ("n_detectors", C.c_int32),
        ("detectors", DetectorDesc * MAX_DETECTORS),
        ("record_interfaces", C.c_int32),
        ("recording_dtype", C.c_int32),
        ("rec_slots", C.c_int32),
        ("rec_store", C.c_void_p),
        ("rec_a", C.c_void_p),
        ("rec_b", C.c_void_p),
        ("rec_w", C.c_void_p),
        ("bloch_axes", C.c_int32),
        ("bloch_cos", C.c_float * 3),
        ("bloch_sin", C.c_float * 3),
        ("n_poles", C.c_int32),
        ("n_disp", C.c_int32),
    ]


class Buffers(C.Structure):
    _fields_ = [
        ("E", C.c_void_p),
        ("H", C.c_void_p),
        ("inv_eps", C.c_void_p),
        ("inv_mu", C.c_void_p),
        ("sigma_E", C.c_void_p),
        ("sigma_H", C.c_void_p),
        ("psi_E", (C.c_void_p * 2) * MAX_SLABS),
        ("psi_H", (C.c_void_p * 2) * MAX_SLABS),
        ("det_state", C.c_void_p * MAX_DETECTORS),
        ("recording", C.c_void_p),
        ("disp_P_curr", C.c_void_p),
        ("disp_P_prev", C.c_void_p),
        ("disp_c1", C.c_void_p),
        ("disp_c2", C.c_void_p),
        ("disp_c3", C.c_void_p),
    ]


class AdjointBuffers(C.Structure):
    _fields_ = [
        ("lam_E", C.c_void_p),
        ("lam_H", C.c_void_p),
        ("lam_psi_E", (C.c_void_p * 2) * MAX_SLABS),
        ("lam_psi_H", (C.c_void_p * 2) * MAX_SLABS),
        ("lam_det", C.c_void_p * MAX_DETECTORS),
        ("grad_inv_eps", C.c_void_p),
        ("grad_inv_mu", C.c_void_p),
        ("lam_P_curr", C.c_void_p),
        ("lam_P_prev", C.c_void_p),
    ]


NOALLOC_SCRATCH_FLOATS = 65536  # FDTD_NOALLOC_SCRATCH_FLOATS

LIB_PATH = Path(__file__).resolve().parent / "libfdtd_gb300.so"
_lib: C.CDLL | None = None

# name -> (restype, argtypes); every symbol include/fdtd_gb300.h declares
SIGNATURES = {
    "fdtd_plan_create": (C.c_int, [C.POINTER(Desc), C.POINTER(C.c_void_p)]),
    "fdtd_plan_destroy": (None, [C.c_void_p]),
    "fdtd_last_error": (C.c_char_p, [C.c_void_p]),
    "fdtd_interface_floats": (C.c_int64, [C.c_void_p]),
    "fdtd_plan_device_bytes": (C.c_int64, [C.c_void_p]),
    "fdtd_footprint_bytes": (C.c_int64, [C.POINTER(Desc)]),
    "fdtd_forward": (C.c_int, [C.c_void_p, C.POINTER(Buffers), C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "fdtd_reverse": (C.c_int, [C.c_void_p, C.POINTER(Buffers), C.c_int32, C.c_int32, C.c_void_p]),
    "fdtd_adjoint": (
        C.c_int,
        [C.c_void_p, C.POINTER(Buffers), C.POINTER(AdjointBuffers), C.c_int32, C.c_int32, C.c_void_p],
    ),
    "fdtd_adjoint_stored": (
        C.c_int,
        [C.c_void_p, C.POINTER(Buffers), C.c_int32, C.c_int32, C.POINTER(AdjointBuffers), C.c_void_p],
    ),
    "fdtd_launches_per_step": (C.c_int32, [C.c_void_p]),
    "fdtd_plan_tune": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "fdtd_plan_tune_shell": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "fdtd_plan_chunk": (C.c_int32, [C.c_void_p]),
    "fdtd_plan_vec": (C.c_int32, [C.c_void_p]),
    "fdtd_plan_tune_tma": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "fdtd_plan_uses_tma": (C.c_int32, [C.c_void_p]),
    "fdtd_plan_tune_shell_tma": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "fdtd_plan_shell_tma": (C.c_int32, [C.c_void_p]),
    "fdtd_plan_status": (C.c_int, [C.c_void_p]),
    "fdtd_debug_inject": (C.c_int, [C.c_int32, C.c_int32]),
    "fdtd_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(Buffers), C.c_int32, C.POINTER(C.c_void_p)]),
    "fdtd_batch_destroy": (None, [C.c_void_p]),
    "fdtd_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "fdtd_batch_forward": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32, C.c_int32, C.c_void_p]),
    "fdtd_batch_tune": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "fdtd_batch_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "fdtd_batch_launches_per_step": (C.c_int32, [C.c_void_p]),
    "fdtd_batch_set_mode": (C.c_int, [C.c_void_p, C.c_int32]),
    "fdtd_batch_mode": (C.c_int32, [C.c_void_p]),
    "fdtd_detector_sample_noalloc": (
        C.c_int,
        [C.POINTER(DetectorDesc), C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.c_void_p, C.c_void_p,
         C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_float, C.c_void_p, C.c_void_p],
    ),
    "fdtd_profile_forward": (
        C.c_int,
        [C.c_void_p, C.POINTER(Buffers), C.c_int32, C.c_int32, C.POINTER(C.c_float), C.c_void_p],
    ),
}


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load the native library, raising if it is absent (there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if build_if_missing:
            from fdtdx_gb300.build import build

            build()
        else:
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m fdtdx_gb300.build` "
                "(the FDTD path runs only on the GPU library)"
            )
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class NativeError(RuntimeError):
    """A status code other than FDTD_OK from the native library (``code`` holds it)."""

    def __init__(self, message: str, code: int | None = None):
        super().__init__(message)
        self.code = code


def check(rc: int, plan: int | None = None, what: str = "") -> None:
    if rc == OK:
        return
    msg = ""
    if plan:
        m = load().fdtd_last_error(plan)
        msg = m.decode() if m else ""
    names = {EINVAL: "FDTD_EINVAL", ENOMEM: "FDTD_ENOMEM", ECUDA: "FDTD_ECUDA", ETIMEOUT: "FDTD_ETIMEOUT",
             ENONFINITE: "FDTD_ENONFINITE"}
    raise NativeError(f"{what}: {names.get(rc, rc)} {msg}".strip(), rc)


def ptr(t) -> int | None:
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return int(t.data_ptr())
