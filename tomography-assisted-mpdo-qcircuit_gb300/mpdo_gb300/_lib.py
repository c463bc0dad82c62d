"""ctypes binding of ``libmpdo_gb300.so`` (the C ABI in include/mpdo_gb300.h).

The library is the only compute path: if it is missing or cannot find a GPU,
every call raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading

from ._build import LIB

MPDO_OK = 0
MPDO_ERR_INVALID = 1
MPDO_ERR_BAD_SHAPE = 2
MPDO_ERR_OOM = 3
MPDO_ERR_CUDA = 4
MPDO_ERR_NOT_CONVERGED = 5
MPDO_ERR_NONFINITE = 6
MPDO_ERR_NO_DEVICE = 7
MPDO_C64 = 0
MPDO_C128 = 1

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)

MPDO_OP_1Q, MPDO_OP_2Q, MPDO_OP_TRUNCATE, MPDO_OP_KAPPA = 1, 2, 3, 4


class Program(C.Structure):
    """``mpdo_program`` of include/mpdo_gb300.h (one circuit of a batch run)."""
    _fields_ = [('n', C.c_int), ('dtype', C.c_int), ('connected', C.c_int), ('vectors', _DP),
                ('chi', C.c_int), ('kappa', C.c_int), ('max_err', C.c_double), ('noisy', C.c_int),
                ('abs_cutoff', C.c_double), ('nops', C.c_int), ('op_kind', _IP), ('op_site', _IP),
                ('op_k', _IP), ('op_offset', C.POINTER(C.c_int64)), ('kraus', _DP), ('z', _DP), ('zz', _DP),
                ('discarded', _DP)]

# name -> (restype, argtypes); mirrors include/mpdo_gb300.h
SIGNATURES = {
    'mpdo_abi_version': (_I, []),
    'mpdo_status_string': (C.c_char_p, [_I]),
    'mpdo_last_error': (C.c_char_p, []),
    'mpdo_engine_create': (_I, [_I, C.POINTER(_P)]),
    'mpdo_engine_destroy': (_I, [_P]),
    'mpdo_engine_set_stream': (_I, [_P, _P]),
    'mpdo_engine_set_option': (_I, [_P, C.c_char_p, _D]),
    'mpdo_engine_sync': (_I, [_P]),
    'mpdo_engine_profile': (_I, [_P, _I]),
    'mpdo_engine_profile_read': (_I, [_P, _I, C.POINTER(C.c_longlong), _DP, _DP, _DP]),
    'mpdo_engine_launch_count': (_I, [_P, C.POINTER(C.c_uint64)]),
    'mpdo_launch_histogram': (_I, [C.c_char_p, _I]),
    'mpdo_chain_create': (_I, [_P, _I, _I, _DP, _I, C.POINTER(_P)]),
    'mpdo_chain_destroy': (_I, [_P]),
    'mpdo_chain_clone': (_I, [_P, C.POINTER(_P)]),
    'mpdo_chain_num_sites': (_I, [_P, _IP]),
    'mpdo_chain_site_dims': (_I, [_P, _I, _IP]),
    'mpdo_chain_bond_present': (_I, [_P, _I, _IP]),
    'mpdo_chain_read_site': (_I, [_P, _I, _DP]),
    'mpdo_chain_write_site': (_I, [_P, _I, _IP, _DP]),
    'mpdo_chain_read_site_device': (_I, [_P, _I, _P]),
    'mpdo_chain_write_site_device': (_I, [_P, _I, _IP, _P]),
    'mpdo_apply_1q': (_I, [_P, _I, _DP, _I]),
    'mpdo_apply_2q': (_I, [_P, _I, _DP, _I, _D]),
    'mpdo_truncate': (_I, [_P, _I, _I, _D, _I, _DP]),
    'mpdo_kappa_truncate': (_I, [_P, _I, _D]),
    'mpdo_qr_left2right': (_I, [_P]),
    'mpdo_svd_right2left': (_I, [_P, _I, _D, _DP]),
    'mpdo_svd_left2right': (_I, [_P, _I, _D, _DP]),
    'mpdo_reduced_dm': (_I, [_P, _IP, _I, _DP]),
    'mpdo_trace_rho_rho': (_I, [_P, _P, _IP, _I, _DP]),
    'mpdo_probs': (_I, [_P, _IP, _I, _DP]),
    'mpdo_expect_ops': (_I, [_P, _IP, _DP, _I, _DP]),
    'mpdo_expect_pauli_batch': (_I, [_P, C.POINTER(C.c_int8), _I, _DP]),
    'mpdo_sample': (_I, [_P, _IP, _I, C.c_int64, C.c_uint64, _D, C.POINTER(C.c_int8)]),
    'mpdo_sample_schemes': (_I, [_P, _IP, _I, _IP, _I, C.c_int64, C.POINTER(C.c_uint64), _D, _DP,
                                 C.POINTER(C.c_int8)]),
    'mpdo_debug_qr': (_I, [_P, _I, _I, _I, _DP, _DP, _DP]),
    'mpdo_debug_svd': (_I, [_P, _I, _I, _I, _DP, _DP, _DP]),
    'mpdo_debug_split': (_I, [_P, _I, _I, _I, _I, _DP, _DP, _DP]),
    'mpdo_keep_count': (_I, [_DP, _I, _I, _I, C.c_double, _I, _IP]),
    'mpdo_right_svd_noalloc': (_I, [_I, _I, _P, _P, _P, _P, _P]),
    'mpdo_batch_create': (_I, [_I, _I, C.POINTER(_P)]),
    'mpdo_batch_destroy': (_I, [_P]),
    'mpdo_batch_set_option': (_I, [_P, C.c_char_p, _D]),
    'mpdo_batch_num_workers': (_I, [_P, _IP]),
    'mpdo_batch_engine': (_I, [_P, _I, C.POINTER(_P)]),
    'mpdo_batch_run': (_I, [_P, _I, C.POINTER(Program), C.POINTER(_P), _IP, _IP]),
    'mpdo_batch_error': (C.c_char_p, [_P, _I]),
    'mpdo_program_grad': (_I, [_P, C.POINTER(Program), _IP, _DP, _D, _D, _DP, _DP, _DP]),
}

_lock = threading.Lock()
_lib = None


class MPDOError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def load() -> C.CDLL:
    """Load the engine library (built by ``mpdo_gb300._build.build``)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB.exists():
                raise RuntimeError(f'{LIB.name} is not built; run mpdo_gb300.build() (needs nvcc)')
            lib = C.CDLL(str(LIB))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(status: int) -> None:
    if status == MPDO_OK:
        return
    lib = load()
    msg = lib.mpdo_last_error().decode(errors='replace') or lib.mpdo_status_string(status).decode()
    if status in (MPDO_ERR_NOT_CONVERGED, MPDO_ERR_NONFINITE):
        import torch
        raise torch.linalg.LinAlgError(msg)
    if status in (MPDO_ERR_INVALID, MPDO_ERR_BAD_SHAPE):
        raise ValueError(msg)
    if status == MPDO_ERR_OOM:
        raise MemoryError(msg)
    raise MPDOError(status, msg)
