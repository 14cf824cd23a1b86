"""ctypes binding of libfmpt (the C ABI declared in include/fmpt.h).

The library is loaded from this package directory.  There is no fallback:
if ``libfmpt.so`` is missing or cannot be loaded, every device entry point
raises ``FMPTError`` (build it with ``finitemptools_gb300.build.build()``).
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfmpt.so")

c_int, c_double, c_void_p, c_int64, c_size_t, c_uint64, c_char_p = (
    ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_int64, ctypes.c_size_t,
    ctypes.c_uint64, ctypes.c_char_p)
P = ctypes.POINTER
dptr = c_void_p        # device pointer
hptr = c_void_p        # host pointer

F64, C128 = 0, 1
PREC = {"fp64": 0, "tf32x3": 1, "tf32": 2, "bf16": 3, "fp64_tc": 4}
TRANS = {"N": 0, "T": 1, "C": 2, "R": 3}


class U1SpaceC(ctypes.Structure):
    """struct fmpt_u1_space: a charge-sorted sector table (nsect, charge*, dim*)."""
    _fields_ = [("nsect", c_int), ("charge", P(c_int)), ("dim", P(c_int))]


SP = P(U1SpaceC)
ip = P(c_int)

STATUS = {0: "ok", -1: "invalid argument", -2: "dimension mismatch", -3: "CUDA error",
          -4: "cuSOLVER error", -5: "device wait timed out", -6: "non-finite value",
          -7: "out of device memory", -8: "unsupported", -9: "not converged"}

# name -> (restype, argtypes); mirrors include/fmpt.h
SIGNATURES = {
    "fmpt_create": (c_int, [c_int, P(c_void_p)]),
    "fmpt_destroy": (c_int, [c_void_p]),
    "fmpt_status_string": (c_char_p, [c_int]),
    "fmpt_last_error": (c_char_p, [c_void_p]),
    "fmpt_synchronize": (c_int, [c_void_p]),
    "fmpt_set_graphs": (c_int, [c_void_p, c_int]),
    "fmpt_set_fused_krylov": (c_int, [c_void_p, c_int]),
    "fmpt_set_cluster_qr": (c_int, [c_void_p, c_int]),
    "fmpt_graph_launch_count": (c_uint64, [c_void_p]),
    "fmpt_set_tuning": (c_int, [c_void_p, c_int]),
    "fmpt_tuning_info": (c_int, [c_void_p, P(c_int), P(c_int64)]),
    "fmpt_op_tile": (c_int, [c_void_p]),
    "fmpt_set_stream": (c_int, [c_void_p, c_void_p]),
    "fmpt_get_stream": (c_void_p, [c_void_p]),
    "fmpt_launch_count": (c_uint64, [c_void_p]),
    "fmpt_version": (c_int, []),
    "fmpt_profile_enable": (c_int, [c_void_p, c_int]),
    "fmpt_profile_read": (c_int, [c_void_p, c_int, P(c_int64), P(c_double)]),
    "fmpt_malloc": (c_int, [c_void_p, c_size_t, P(c_void_p)]),
    "fmpt_free": (c_int, [c_void_p, c_void_p]),
    "fmpt_memcpy_h2d": (c_int, [c_void_p, dptr, hptr, c_size_t]),
    "fmpt_memcpy_d2h": (c_int, [c_void_p, hptr, dptr, c_size_t]),
    "fmpt_memcpy_d2d": (c_int, [c_void_p, dptr, dptr, c_size_t]),
    "fmpt_memset_zero": (c_int, [c_void_p, dptr, c_size_t]),
    "fmpt_gemm": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, hptr, dptr, c_int,
                          dptr, c_int, hptr, dptr, c_int]),
    "fmpt_dot": (c_int, [c_void_p, c_int, c_int64, dptr, dptr, hptr]),
    "fmpt_nrm2": (c_int, [c_void_p, c_int, c_int64, dptr, hptr]),
    "fmpt_axpy": (c_int, [c_void_p, c_int, c_int64, hptr, dptr, dptr]),
    "fmpt_scal": (c_int, [c_void_p, c_int, c_int64, hptr, dptr]),
    "fmpt_scale_dim": (c_int, [c_void_p, c_int, c_int, c_int, c_int, dptr, dptr]),
    "fmpt_ac2_prime": (c_int, [c_void_p, c_int, c_int, dptr, hptr, hptr, dptr, dptr, dptr,
                               c_int, c_int, c_int, c_int, c_int, c_int, c_int]),
    "fmpt_ac_prime": (c_int, [c_void_p, c_int, c_int, dptr, hptr, dptr, dptr, dptr,
                              c_int, c_int, c_int, c_int, c_int]),
    "fmpt_ac2_prime_noalloc": (c_int, [c_void_p, c_int, dptr, hptr, hptr, dptr, dptr, dptr,
                                       c_int, c_int, c_int, c_int, c_int, c_int, c_int]),
    "fmpt_c_prime": (c_int, [c_void_p, c_int, c_int, dptr, dptr, dptr, dptr, c_int, c_int, c_int]),
    "fmpt_updateleft": (c_int, [c_void_p, c_int, c_int, dptr, dptr, hptr, dptr, dptr,
                                c_int, c_int, c_int, c_int, c_int]),
    "fmpt_updateright": (c_int, [c_void_p, c_int, c_int, dptr, dptr, hptr, dptr, dptr,
                                 c_int, c_int, c_int, c_int, c_int]),
    "fmpt_op_ac2": (c_int, [c_void_p, c_int, c_int, hptr, hptr, dptr, dptr, c_int, c_int, c_int,
                            c_int, c_int, c_int, c_int, P(c_void_p)]),
    "fmpt_op_ac": (c_int, [c_void_p, c_int, c_int, hptr, dptr, dptr, c_int, c_int, c_int, c_int,
                           c_int, P(c_void_p)]),
    "fmpt_op_c": (c_int, [c_void_p, c_int, c_int, dptr, dptr, c_int, c_int, c_int, P(c_void_p)]),
    "fmpt_op_apply": (c_int, [c_void_p, dptr, dptr]),
    "fmpt_op_size": (c_int64, [c_void_p]),
    "fmpt_op_destroy": (c_int, [c_void_p]),
    "fmpt_op_set_projectors": (c_int, [c_void_p, c_int, P(c_void_p)]),
    "fmpt_set_svd_method": (c_int, [c_void_p, c_int]),
    "fmpt_set_tc_tile": (c_int, [c_void_p, c_int]),
    "fmpt_set_f64_engine": (c_int, [c_void_p, c_int]),
    "fmpt_set_wait_test": (c_int, [c_void_p, c_int64, c_int]),
    "fmpt_ac2_prime_host": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                    c_int, c_int, c_int]),
    "fmpt_apply_gate": (c_int, [c_void_p, c_int, c_void_p, c_int, dptr, dptr, c_int, c_int]),
    "fmpt_eigsolve": (c_int, [c_void_p, dptr, c_int, c_int, c_int, c_double, c_int, P(c_double),
                              dptr, P(c_double), P(c_int), P(c_int)]),
    "fmpt_lanczos_ground": (c_int, [c_void_p, dptr, c_int, c_double, c_int, P(c_double), dptr,
                                    P(c_int), P(c_int)]),
    "fmpt_dmrg2_sweep": (c_int, [c_void_p, c_int, c_int, c_int, c_int, P(c_int), P(c_int),
                                 P(c_void_p), P(c_int64), P(c_void_p), P(c_int64), P(c_void_p),
                                 P(c_int), P(c_void_p), c_int, c_double, c_int, c_double, c_int,
                                 c_int, P(c_double), P(c_double)]),
    "fmpt_exponentiate": (c_int, [c_void_p, c_double, c_double, dptr, dptr, c_int, c_double,
                                  P(c_int)]),
    "fmpt_svd_trunc": (c_int, [c_void_p, c_int, dptr, c_int, c_int, c_int, c_double, dptr, dptr,
                               dptr, P(c_int), P(c_double)]),
    "fmpt_dm_split": (c_int, [c_void_p, c_int, dptr, c_int, c_int, c_int, c_double, c_int,
                              dptr, dptr, dptr, P(c_int), P(c_double)]),
    "fmpt_qr": (c_int, [c_void_p, c_int, dptr, c_int, c_int, dptr, dptr]),
    "fmpt_lq": (c_int, [c_void_p, c_int, dptr, c_int, c_int, dptr, dptr]),
    "fmpt_expm_nodes": (c_int, [c_void_p, c_double, c_double, dptr, c_int, c_int, P(c_double),
                                dptr, P(c_double)]),
    "fmpt_wgrad": (c_int, [c_void_p, c_int, dptr, dptr, dptr, dptr, dptr, c_int, c_int, c_int,
                           c_int, c_int]),
    "fmpt_swap13": (c_int, [c_void_p, c_int, dptr, dptr, c_int, c_int, c_int, c_int]),
    "fmpt_copy2d": (c_int, [c_void_p, c_int, c_int, c_int, dptr, c_int64, c_int64, dptr, c_int64,
                            c_int64]),
    "fmpt_qr_adjoint": (c_int, [c_void_p, c_int, dptr, dptr, dptr, dptr, dptr, c_int, c_int]),
    "fmpt_u1_twosite_size": (c_int, [c_void_p, SP, SP, c_int, ip, c_int, ip, P(c_int64)]),
    "fmpt_u1_pack2": (c_int, [c_void_p, c_int, dptr, dptr, SP, SP, c_int, ip, c_int, ip, c_int]),
    "fmpt_u1_op_ac2": (c_int, [c_void_p, c_int, hptr, hptr, dptr, dptr, SP, SP, c_int, ip, c_int,
                               ip, c_int, ip, c_int, ip, c_int, ip, P(c_void_p)]),
    "fmpt_op_flops": (c_int, [c_void_p, P(c_double)]),
    "fmpt_u1_twosite": (c_int, [c_void_p, c_int, dptr, dptr, dptr, SP, SP, SP, c_int, ip, c_int,
                                ip]),
    "fmpt_u1_updateleft": (c_int, [c_void_p, c_int, dptr, dptr, hptr, dptr, dptr, SP, SP, c_int,
                                   ip, c_int, ip, c_int, ip]),
    "fmpt_u1_updateright": (c_int, [c_void_p, c_int, dptr, dptr, hptr, dptr, dptr, SP, SP, c_int,
                                    ip, c_int, ip, c_int, ip]),
    "fmpt_u1_split": (c_int, [c_void_p, c_int, dptr, SP, SP, c_int, ip, c_int, ip, c_int,
                              c_double, c_int, c_int, dptr, dptr, dptr, c_int, ip, ip, ip,
                              P(c_double)]),
}


class FMPTError(RuntimeError):
    """A libfmpt call returned a non-zero status (the reference would throw
    DimensionMismatch / ArgumentError / an exception from LAPACK)."""

    def __init__(self, status, msg):
        super().__init__("libfmpt status %d (%s): %s" % (status, STATUS.get(status, "?"), msg))
        self.status = status


_lib = None
_lock = threading.Lock()


def lib():
    """The loaded libfmpt (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise FMPTError(-8, "libfmpt.so is not built (run finitemptools_gb300.build.build())")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status, handle=None):
    if status != 0:
        msg = ""
        if handle is not None:
            m = lib().fmpt_last_error(handle)
            msg = m.decode() if m else ""
        raise FMPTError(status, msg)
    return status
