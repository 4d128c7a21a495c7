"""ctypes binding of ``libpynof_gb300.so`` (the C ABI in ``include/pynof_gb300.h``).

The library is loaded from the package directory.  There is no fallback: if
the library is missing or fails to load, every call raises, so no silent CPU
path can stand in for the CUDA kernels.
"""
from __future__ import annotations

import ctypes
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libpynof_gb300.so")

GB_OK = 0
STATUS_NAMES = {
    1: "GB_ERR_INVALID_ARG",
    2: "GB_ERR_BAD_SHAPE",
    3: "GB_ERR_WORKSPACE",
    4: "GB_ERR_CUDA",
    5: "GB_ERR_TIMEOUT",
    6: "GB_ERR_NONFINITE",
    7: "GB_ERR_UNSUPPORTED",
}

_c = ctypes
_P = _c.c_void_p
_I = _c.c_int
_Z = _c.c_size_t

#: name -> (restype, argtypes).  Every entry is declared in include/pynof_gb300.h.
SIGNATURES = {
    "gb_last_error": (_c.c_char_p, []),
    "gb_version": (_I, []),
    "gb_profile_start": (_I, []),
    "gb_profile_stop": (_I, [_c.c_char_p, _Z]),
    "gb_check_symmetric_f64": (_I, [_P, _I, _I, _P, _P]),
    "gb_jkj_ri_workspace_f64": (_Z, [_I, _I, _I]),
    "gb_jkj_ri_f64": (_I, [_P, _P, _I, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_jkj_ri_noalloc_f64": (_I, [_P, _P, _I, _I, _I, _P, _P, _P]),
    "gb_jkh_mo_ri_workspace_f64": (_Z, [_I, _I, _I]),
    "gb_jkh_mo_ri_f64": (_I, [_P, _P, _P, _I, _I, _I, _P, _P, _P, _P, _Z, _P]),
    "gb_mo_ri_workspace_f64": (_Z, [_I, _I, _I]),
    "gb_mo_ri_f64": (_I, [_P, _P, _P, _I, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_lagrange2_ri_workspace_f64": (_Z, [_I, _I, _I]),
    "gb_lagrange2_ri_f64": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_jkj_full_workspace_f64": (_Z, [_I, _I]),
    "gb_jkj_full_f64": (_I, [_P, _P, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_jkh_mo_full_workspace_f64": (_Z, [_I, _I]),
    "gb_jkh_mo_full_f64": (_I, [_P, _P, _P, _I, _I, _P, _P, _P, _P, _Z, _P]),
    "gb_mo_full_workspace_f64": (_Z, [_I, _I]),
    "gb_mo_full_f64": (_I, [_P, _P, _P, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_lagrange2_full_workspace_f64": (_Z, [_I, _I]),
    "gb_lagrange2_full_f64": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_fock_rc_workspace_f64": (_Z, [_I, _I]),
    "gb_fock_rc_f64": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_fock_ro_workspace_f64": (_Z, [_I, _I]),
    "gb_fock_ro_f64": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_lagrange_workspace_f64": (_Z, [_I, _I]),
    "gb_lagrange_f64": (_I, [_P, _P, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_energy_elec_workspace_f64": (_Z, [_I, _I]),
    "gb_energy_elec_f64": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_ri_factor_f64": (_I, [_P, _P, _I, _I, _P, _P]),
    "gb_dgemm_f64": (_I, [_P, _P, _I, _I, _I, _P, _P]),
    "gb_mo4_full_workspace_f64": (_Z, [_I, _I, _I, _I]),
    "gb_mo4_full_f64": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_graph_begin": (_I, [_P]),
    "gb_graph_end": (_I, [_P, _P]),
    "gb_graph_launch": (_I, [_P, _P]),
    "gb_graph_destroy": (_I, [_P]),
    "gb_density_hf_f64": (_I, [_P, _I, _I, _I, _P, _P]),
    "gb_jk_hf_full_workspace_f64": (_Z, [_I]),
    "gb_jk_hf_full_f64": (_I, [_P, _P, _I, _P, _P, _P, _Z, _P]),
    "gb_rotate_orbital_workspace_f64": (_Z, [_I]),
    "gb_rotate_orbital_f64": (_I, [_P, _P, _I, _I, _c.c_double, _P, _P, _Z, _P]),
    "gb_occ_energy_grad_f64": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _P, _P]),
    "gb_calce_f64": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _P]),
    "gb_occ_workspace_bytes": (_Z, [_I, _I, _I]),
    "gb_occ_minimize_dev": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _c.c_double, _I, _P, _P, _P, _P, _P, _P, _Z, _P]),
    "gb_occ_minimize_dev_sync": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _c.c_double, _I, _P, _P, _P, _P, _P, _P, _Z,
                                      _P]),
    "gb_occ_energy_grad_dev": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_occ_release": (_I, [_P]),
    "gb_device_status": (_I, [_I, _c.POINTER(_I)]),
    "gb_set_wait_limit_ns": (_I, [_c.c_ulonglong]),
    "gb_test_withhold_stage": (_I, [_I]),
    "gb_dgemm_mixed_workspace": (_Z, [_I, _I, _I, _I]),
    "gb_dgemm_mixed": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_ri_prepare_bytes_mixed": (_Z, [_I, _I, _I]),
    "gb_ri_prepare_mixed": (_I, [_P, _I, _I, _I, _P, _Z, _P]),
    "gb_jkj_ri_workspace_mixed": (_Z, [_I, _I, _I, _I]),
    "gb_jkj_ri_mixed": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_jkj_ri_mixed_j": (_I, [_P, _P, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_jkj_ri_mixed_k": (_I, [_I, _I, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_jkj_ri_mixed_t": (_I, [_P, _P, _I, _I, _I, _I, _P, _Z, _P]),
    "gb_jkj_ri_mixed_jr": (_I, [_P, _I, _I, _I, _I, _I, _I, _P, _P, _Z, _P]),
    "gb_jkj_batch_workspace_mixed": (_Z, [_I, _P, _P, _P, _I]),
    "gb_jkj_batch_create_mixed": (_I, [_I, _P, _P, _P, _P, _P, _I, _P, _P, _P, _P, _Z, _P, _P]),
    "gb_batch_launch": (_I, [_P, _P]),
    "gb_batch_destroy": (_I, [_P]),
    "gb_jkh_mo_ri_workspace_mixed": (_Z, [_I, _I, _I, _I]),
    "gb_jkh_mo_ri_mixed": (_I, [_P, _P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _Z, _P]),
    "gb_lagrange2_ri_workspace_mixed": (_Z, [_I, _I, _I, _I]),
    "gb_lagrange2_ri_mixed": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P, _P, _Z, _P]),
    "gb_jkh_lagrange2_ri_workspace_mixed": (_Z, [_I, _I, _I, _I]),
    "gb_jkh_lagrange2_ri_mixed": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _Z,
                                       _P]),
}

_lock = threading.Lock()
_lib = None


class GBError(RuntimeError):
    """A libpynof_gb300 call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load(path: str = LIB_PATH):
    """Load the library once and attach the declared signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"libpynof_gb300.so not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != GB_OK:
        msg = load().gb_last_error().decode(errors="replace")
        if status in (2, 1):
            raise GBError(status, msg)
        raise GBError(status, msg)


def call(name: str, *args) -> None:
    """Call a status-returning entry point and raise GBError on failure."""
    check(getattr(load(), name)(*args))


def query(name: str, *args) -> int:
    return int(getattr(load(), name)(*args))


def device_status(reset: bool = True) -> int:
    """Status word of the tensor-core kernels (0 = ok); synchronises the device."""
    v = _c.c_int(0)
    call("gb_device_status", 1 if reset else 0, _c.byref(v))
    return int(v.value)


def profile_start() -> None:
    call("gb_profile_start")


def profile_stop() -> dict:
    """{kernel: (launches, total_ms)} since profile_start()."""
    import json

    buf = ctypes.create_string_buffer(1 << 16)
    call("gb_profile_stop", buf, len(buf))
    return {k: (int(v[0]), float(v[1])) for k, v in json.loads(buf.value.decode()).items()}
