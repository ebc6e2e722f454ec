"""ctypes binding of ``libqca_gb300.so`` (the C ABI of ``include/qca_gb300.h``).

The library is built in-tree by ``build.py``.  Loading fails loudly when it is
missing: there is no CPU fallback for any operation of this package.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqca_gb300.so")

QCA_OK = 0
QCA_ERR_INVALID = 1
QCA_ERR_CUDA = 2
QCA_ERR_OOM = 3
QCA_ERR_BREAKDOWN = 4
QCA_ERR_NOT_CONVERGED = 5
QCA_ERR_NAN = 6
QCA_ERR_ADMISSION = 7
QCA_ERR_NO_DEVICE = 8

QCA_PREC_FP64 = 0
QCA_PREC_MIXED = 1
QCA_ALGO_1TDVP = 1
QCA_ALGO_2TDVP = 2
QCA_ALGO_A1TDVP = 3

_ERROR_NAMES = {
    QCA_ERR_INVALID: "invalid argument",
    QCA_ERR_CUDA: "CUDA error",
    QCA_ERR_OOM: "out of device memory",
    QCA_ERR_BREAKDOWN: "Krylov breakdown",
    QCA_ERR_NOT_CONVERGED: "iteration did not converge",
    QCA_ERR_NAN: "non-finite value",
    QCA_ERR_ADMISSION: "device-memory budget exceeded",
    QCA_ERR_NO_DEVICE: "no CUDA device",
}


class QcaError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, code: int, message: str) -> None:
        super().__init__(f"{_ERROR_NAMES.get(code, 'error')} ({code}): {message}")
        self.code = code


class AdmissionError(QcaError):
    pass


class ChainDesc(ctypes.Structure):
    _fields_ = [
        ("n_sites", ctypes.c_int),
        ("mpo_bonds", ctypes.POINTER(ctypes.c_int)),
        ("mpo", ctypes.POINTER(ctypes.c_double)),
        ("mps_bonds", ctypes.POINTER(ctypes.c_int)),
        ("mps", ctypes.POINTER(ctypes.c_double)),
        ("algorithm", ctypes.c_int),
        ("max_bond_dim", ctypes.c_int),
        ("svd_epsilon", ctypes.c_double),
        ("step_size", ctypes.c_double),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_PD = ctypes.POINTER(ctypes.c_double)
_PI = ctypes.POINTER(ctypes.c_int)
_SZ = ctypes.c_size_t

# name -> argtypes (all return int status except qca_last_error / qca_version)
SIGNATURES = {
    "qca_device_count": [_PI],
    "qca_exact_create": [_I, _I, _I, _I, _I, _I, ctypes.POINTER(_P)],
    "qca_exact_destroy": [_P],
    "qca_exact_set_state": [_P, _PD, _P],
    "qca_exact_set_state_device": [_P, _P, _P],
    "qca_exact_get_state": [_P, _PD, _P],
    "qca_exact_state_device": [_P, ctypes.POINTER(_P)],
    "qca_exact_step": [_P, _D, _I, _P],
    "qca_exact_measure": [_P, _PD, _PD, _P],
    "qca_exact_footprint": [_I, _I, _I, ctypes.POINTER(_SZ)],
    "qca_exact_step_noalloc": [_I, _I, _I, _I, _I, _D, _I, _P, _P, _P],
    "qca_engine_create": [_I, _SZ, ctypes.POINTER(_P)],
    "qca_engine_destroy": [_P],
    "qca_chain_footprint": [ctypes.POINTER(ChainDesc), _I, ctypes.POINTER(_SZ)],
    "qca_chain_add": [_P, ctypes.POINTER(ChainDesc), _P, _PI],
    "qca_chain_remove": [_P, _I],
    "qca_engine_step": [_P, _I, _P],
    "qca_engine_step_chains": [_P, _PI, _I, _I, _P],
    "qca_chain_schedule": [_P, _I, _I],
    "qca_engine_advance": [_P, _PI, _I, _I, _P],
    "qca_chain_progress": [_P, _I, ctypes.POINTER(ctypes.c_longlong)],
    "qca_chain_measure": [_P, _I, _PD, _PD, _PD, _PD, _P],
    "qca_engine_measure": [_P, _PI, _I, _PD, _PD, _PD, _PD, _P],
    "qca_chain_bonds": [_P, _I, _PI],
    "qca_chain_get_mps": [_P, _I, _PD, _SZ, _P],
    "qca_chain_stats": [_P, _I, _PD],
    "qca_chain_stats_ex": [_P, _I, _PD, _I],
    "qca_engine_profile": [_P, _I],
    "qca_engine_kernel_stats": [_P, _PD, _I],
    "qca_test_gemm_c64": [_I, _I, _I, _P, _P, _P, _I, _P],
    "qca_test_svd": [_I, _I, _I, _P, _I, _D, _P, _P, _P, _PI, _P],
    "qca_test_svd_sweeps": [_I, _I, _I, _P, _I, _D, _I, _P, _P, _P, _PI, _P],
}

_lib = None
_lock = threading.Lock()


def load() -> ctypes.CDLL:
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(LIB_PATH)
        lib.qca_last_error.restype = ctypes.c_char_p
        lib.qca_last_error.argtypes = []
        lib.qca_version.restype = ctypes.c_int
        lib.qca_version.argtypes = []
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != QCA_OK:
        msg = load().qca_last_error().decode(errors="replace")
        if status == QCA_ERR_ADMISSION:
            raise AdmissionError(status, msg)
        raise QcaError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def device_count() -> int:
    n = ctypes.c_int(0)
    call("qca_device_count", ctypes.byref(n))
    return n.value


def as_ptr(arr, ctype=ctypes.c_double):
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


def stream_handle(stream) -> ctypes.c_void_p:
    """Accept None, an int handle, or a torch.cuda.Stream."""
    if stream is None:
        return ctypes.c_void_p(0)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(int(stream.cuda_stream))
