"""Dense device linear algebra used around the hot path: GEMM plumbing,
truncated SVD with MPSTruncation semantics, QR/LQ gauge moves, BLAS-1.

Mirrors auxiliary/truncation.jl, auxiliary/stable_svd.jl and the
TensorKit leftorth!/rightorth calls of the reference.
"""

import ctypes

import numpy as np

from ._native import C128, TRANS, lib
from .device import DeviceTensor

__all__ = ["MPSTruncation", "DefaultSVDCutoff", "default_truncation", "gemm", "matmul",
           "dot", "norm", "scal", "axpy", "stable_tsvd", "dm_split", "leftorth", "rightorth",
           "scale_rows", "scale_cols"]

DefaultSVDCutoff = 1.0e-8       # auxiliary/truncation.jl:49
DefaultNonSymmetricD = 100      # auxiliary/truncation.jl:51


class MPSTruncation:
    """auxiliary/truncation.jl:8-16: truncate singular values below eps*||s||_2
    first, then keep at most D."""

    def __init__(self, D, eps=DefaultSVDCutoff, verbosity=1):
        self.D = int(D)
        self.eps = float(eps)
        self.verbosity = int(verbosity)

    def __repr__(self):
        return "MPSTruncation(D=%d, eps=%g)" % (self.D, self.eps)


def default_truncation():
    """default_truncation() (truncation.jl:75): D=100, cutoff 1e-8."""
    return MPSTruncation(DefaultNonSymmetricD, DefaultSVDCutoff)


def _c2(z):
    return (ctypes.c_double * 2)(float(np.real(z)), float(np.imag(z)))


def gemm(A, B, out_shape, m, n, k, ta="N", tb="N", alpha=1.0, beta=0.0, C=None, lda=None,
         ldb=None, ldc=None):
    """C = alpha op(A) op(B) + beta C on device tensors viewed as matrices."""
    h = A.h
    dt = np.complex128 if (A.code == C128 or B.code == C128) else np.float64
    if C is None:
        C = DeviceTensor(out_shape, dt, h)
    if (A.code != C.code) or (B.code != C.code):
        raise TypeError("gemm: mixed real/complex operands")
    an = ta in ("N", "R")
    bn = tb in ("N", "R")
    lda = lda or (m if an else k)
    ldb = ldb or (k if bn else n)
    ldc = ldc or m
    h.check(lib().fmpt_gemm(h.ptr, C.code, TRANS[ta], TRANS[tb], m, n, k, _c2(alpha), A.ptr, lda,
                            B.ptr, ldb, _c2(beta), C.ptr, ldc))
    return C


def matmul(A, B, ta="N", tb="N"):
    """op(A) @ op(B) for 2-D device tensors."""
    am, ak = A.shape if ta in ("N", "R") else A.shape[::-1]
    bk, bn = B.shape if tb in ("N", "R") else B.shape[::-1]
    if ak != bk:
        raise ValueError("DimensionMismatch")
    return gemm(A, B, (am, bn), am, bn, ak, ta, tb, lda=A.shape[0], ldb=B.shape[0])


def dot(x, y):
    """<x, y> = sum conj(x) y (Julia dot)."""
    out = (ctypes.c_double * 2)()
    x.h.check(lib().fmpt_dot(x.h.ptr, x.code, x.size, x.ptr, y.ptr, out))
    return complex(out[0], out[1]) if x.code == C128 else out[0]


def norm(x):
    out = (ctypes.c_double * 1)()
    x.h.check(lib().fmpt_nrm2(x.h.ptr, x.code, x.size, x.ptr, out))
    return out[0]


def scal(a, x):
    x.h.check(lib().fmpt_scal(x.h.ptr, x.code, x.size, _c2(a), x.ptr))
    return x


def axpy(a, x, y):
    y.h.check(lib().fmpt_axpy(y.h.ptr, y.code, y.size, _c2(a), x.ptr, y.ptr))
    return y


def scale_rows(M, m, n, s):
    """M[i, j] *= s[i]; s is a real device vector."""
    M.h.check(lib().fmpt_scale_dim(M.h.ptr, M.code, 0, m, n, s.ptr, M.ptr))
    return M


def scale_cols(M, m, n, s):
    """M[i, j] *= s[j]."""
    M.h.check(lib().fmpt_scale_dim(M.h.ptr, M.code, 1, m, n, s.ptr, M.ptr))
    return M


def stable_tsvd(M, m, n, trunc=None):
    """stable_tsvd!(m; trunc) (auxiliary/stable_svd.jl:12-18) of a device
    tensor viewed as an m x n matrix.  Returns (U [m,k], S [k] real, Vt [k,n],
    err); without ``trunc`` nothing is dropped."""
    h = M.h
    r = min(m, n)
    U = DeviceTensor((m, r), M.dtype, h)
    S = DeviceTensor((r,), np.float64, h)
    Vt = DeviceTensor((r, n), M.dtype, h)
    k = ctypes.c_int()
    err = ctypes.c_double()
    maxD = trunc.D if trunc is not None else r
    eps = trunc.eps if trunc is not None else 0.0
    h.check(lib().fmpt_svd_trunc(h.ptr, M.code, M.ptr, m, n, maxD, eps, U.ptr, S.ptr, Vt.ptr,
                                 ctypes.byref(k), ctypes.byref(err)))
    k = k.value
    U.view_as((m, k))
    S.view_as((k,))
    Vt.view_as((k, n))
    return U, S, Vt, err.value


def dm_split(M, m, n, trunc, side):
    """Truncated split through the reduced density matrix (White's DMRG
    truncation, FP64 on the device).  side 0: returns (U [m,k] orthonormal,
    S [k], SV = U^H M [k,n], err); side 1: (US = M V [m,k], S [k], V^H [k,n]
    orthonormal, err).  Same truncation rule as stable_tsvd."""
    h = M.h
    r = min(m, n)
    Aout = DeviceTensor((m, r), M.dtype, h)
    S = DeviceTensor((r,), np.float64, h)
    Bout = DeviceTensor((r, n), M.dtype, h)
    k = ctypes.c_int()
    err = ctypes.c_double()
    h.check(lib().fmpt_dm_split(h.ptr, M.code, M.ptr, m, n, trunc.D, trunc.eps, int(side),
                                Aout.ptr, S.ptr, Bout.ptr, ctypes.byref(k), ctypes.byref(err)))
    k = k.value
    return Aout.view_as((m, k)), S.view_as((k,)), Bout.view_as((k, n)), err.value


def leftorth(M, m, n):
    """leftorth!(M, alg=QR()): M (m x n) = Q (m x r) R (r x n)."""
    h = M.h
    r = min(m, n)
    Q = DeviceTensor((m, r), M.dtype, h)
    R = DeviceTensor((r, n), M.dtype, h)
    h.check(lib().fmpt_qr(h.ptr, M.code, M.ptr, m, n, Q.ptr, R.ptr))
    return Q, R


def rightorth(M, m, n):
    """rightorth(M, alg=LQ()): M (m x n) = L (m x r) Q (r x n)."""
    h = M.h
    r = min(m, n)
    Lm = DeviceTensor((m, r), M.dtype, h)
    Q = DeviceTensor((r, n), M.dtype, h)
    h.check(lib().fmpt_lq(h.ptr, M.code, M.ptr, m, n, Lm.ptr, Q.ptr))
    return Lm, Q
