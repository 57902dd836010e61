"""
ctypes binding of the C ABI in ``include/tad_dftd4_gb300.h``.

The structures below mirror the header field by field.  The library is
loaded from the package's ``_lib`` directory; if it is missing the import of
any compute entry point fails with a clear error (there is no CPU fallback).
"""

from __future__ import annotations

import ctypes
from ctypes import c_double, c_int, c_int32, c_size_t, c_uint32, c_void_p, c_char_p
from pathlib import Path

from . import _build

ABI_VERSION = 2
NREF = 7
NFREQ = 23

D4_OK = 0
STATUS_NAMES = {
    0: "D4_OK",
    1: "D4_ERR_ARGUMENT",
    2: "D4_ERR_WORKSPACE",
    3: "D4_ERR_CUDA",
    4: "D4_ERR_ELEMENT",
    5: "D4_ERR_EEQ_SINGULAR",
    6: "D4_ERR_NONFINITE",
    7: "D4_ERR_TOO_MANY_ELEMENTS",
    8: "D4_ERR_DEVICE_TIMEOUT",
}

MODEL_D4 = 0
MODEL_D4S = 1

FLAG_GRADIENT = 1
FLAG_CHARGES_IN = 2
FLAG_MIXED = 4
FLAG_PARAM_GRAD = 8
FLAG_EXACT_C9 = 16
FLAG_NO_HOST_WAIT = 32  # the multi-CTA EEQ never waits for the stream inside a call
FLAG_TEST_TIMEOUT = 0x80000000  # test hook: the pair kernel's first MMA wait counts as timed out
PARAM_GRAD_STRIDE = 12  # D4_PARAM_GRAD_STRIDE: s6 s8 s10 a1 a2 s9 alp rs6 rs8 bet - -

DAMP_RATIONAL = 0
DAMP_ZERO = 1
DAMP_MZERO = 2
DAMP_OP = 3
STATUS_OFFSET = 0  # D4_STATUS_OFFSET: byte offset of the device status word in a workspace


class Tables(ctypes.Structure):
    _fields_ = [
        ("n_ref_elem", c_int32),
        ("n_elem", c_int32),
        ("alpha", c_void_p),
        ("refcovcn", c_void_p),
        ("refc", c_void_p),
        ("refq", c_void_p),
        ("gam", c_void_p),
        ("zeff", c_void_p),
        ("r4r2", c_void_p),
        ("cov_d3", c_void_p),
        ("en", c_void_p),
        ("eeq_chi", c_void_p),
        ("eeq_eta", c_void_p),
        ("eeq_kcn", c_void_p),
        ("eeq_rad", c_void_p),
        ("wfpair", c_void_p),
        ("freq_weights", c_void_p),
    ]


class ModelCfg(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("ga", c_double), ("gc", c_double), ("wf", c_double)]


class Params(ctypes.Structure):
    _fields_ = [
        ("s6", c_double),
        ("s8", c_double),
        ("s10", c_double),
        ("a1", c_double),
        ("a2", c_double),
        ("s9", c_double),
        ("alp", c_double),
        ("has_s8", c_int32),
        ("has_s10", c_int32),
        ("cut_disp2", c_double),
        ("cut_disp3", c_double),
        ("cut_cn", c_double),
        ("cut_cn_eeq", c_double),
        ("cn_eeq_max", c_double),
        ("kcn", c_double),
        ("k4", c_double),
        ("k5", c_double),
        ("k6", c_double),
        ("damping", c_int32),
        ("reserved", c_int32),
        ("rs6", c_double),
        ("rs8", c_double),
        ("bet", c_double),
    ]


class Batch(ctypes.Structure):
    _fields_ = [
        ("n_struct", c_int32),
        ("n_pad", c_int32),
        ("d_numbers", c_void_p),
        ("d_positions", c_void_p),
        ("d_charge", c_void_p),
        ("d_charges_in", c_void_p),
        ("d_r4r2_in", c_void_p),
        ("d_energy_weights", c_void_p),
        ("d_rvdw_in", c_void_p),
    ]


class Outputs(ctypes.Structure):
    _fields_ = [
        ("d_energy", c_void_p),
        ("d_gradient", c_void_p),
        ("d_charges", c_void_p),
        ("d_cn", c_void_p),
        ("d_param_grad", c_void_p),
        ("d_cn_eeq", c_void_p),
    ]


class Properties(ctypes.Structure):
    _fields_ = [
        ("d_cn", c_void_p),
        ("d_charges", c_void_p),
        ("d_c6", c_void_p),
        ("d_alpha", c_void_p),
    ]


# name -> (restype, argtypes) of every exported function
SIGNATURES = {
    "d4_abi_version": (c_int, []),
    "d4_status_string": (c_char_p, [c_int]),
    "d4_last_cuda_error": (c_char_p, []),
    "d4_prepare_alpha": (
        c_int,
        [ctypes.POINTER(Tables), ctypes.POINTER(ModelCfg), c_void_p, c_void_p, c_void_p,
         c_void_p, c_void_p, c_void_p, c_int32, c_void_p, c_void_p, c_void_p],
    ),
    "d4_workspace_size": (c_size_t, [c_int32, c_int32, c_int32, c_uint32]),
    "d4_dispersion": (
        c_int,
        [ctypes.POINTER(Tables), ctypes.POINTER(ModelCfg), ctypes.POINTER(Batch),
         ctypes.POINTER(Params), c_uint32, c_int32, c_void_p, c_size_t,
         ctypes.POINTER(Outputs), c_void_p],
    ),
    "d4_read_status": (c_int, [c_void_p, c_void_p]),
    "d4_eeq_residuals": (c_int, [c_void_p, c_int32, c_void_p, c_void_p]),
    "d4_status_async": (c_int, [c_void_p, c_void_p, c_void_p]),
    "d4_timing_begin": (c_int, [c_int32]),
    "d4_timing_end": (c_int, [ctypes.POINTER(ctypes.c_float), c_int32,
                              ctypes.POINTER(c_int32)]),
    "d4_stage_count": (c_int32, []),
    "d4_stage_name": (c_char_p, [c_int32]),
    "d4_probe_fma": (c_int, [c_int32, c_int32, c_int32, c_void_p,
                             ctypes.POINTER(ctypes.c_float), c_void_p]),
    "d4_properties": (
        c_int,
        [ctypes.POINTER(Tables), ctypes.POINTER(ModelCfg), ctypes.POINTER(Batch),
         ctypes.POINTER(Params), c_void_p, c_size_t, ctypes.POINTER(Properties), c_void_p],
    ),
    "d4_selftest_wait": (c_int, [c_void_p, ctypes.c_uint64, c_void_p]),
    "d4_dispersion_noalloc": (
        c_int,
        [ctypes.POINTER(Tables), ctypes.POINTER(ModelCfg), ctypes.POINTER(Batch),
         ctypes.POINTER(Params), c_uint32, c_int32, ctypes.POINTER(Outputs), c_int32,
         c_void_p],
    ),
}

_LIB: ctypes.CDLL | None = None


class LibraryError(RuntimeError):
    """The compiled library is missing or failed."""


def library_path() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the shared library (building it first when it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists() or (build_if_missing and not _build.up_to_date()):
        if not build_if_missing:
            raise LibraryError(f"CUDA library not built: {path}")
        try:
            _build.build()
        except Exception as exc:  # pragma: no cover - depends on toolchain
            raise LibraryError(f"cannot build the CUDA library: {exc}") from exc
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.d4_abi_version() != ABI_VERSION:
        raise LibraryError("ABI version mismatch between library and binding")
    _LIB = lib
    return lib


def check(status: int, what: str) -> None:
    """Raise for a non-zero status code."""
    if status == D4_OK:
        return
    lib = load()
    msg = lib.d4_status_string(status).decode()
    if status == 3:
        msg += f" ({lib.d4_last_cuda_error().decode()})"
    raise LibraryError(f"{what}: {STATUS_NAMES.get(status, status)}: {msg}")
