"""Environment transfer updates (mpo/transfer.jl:26-55,
mpohamiltonian/transfer.jl:48-75) on device tensors."""

import ctypes

import numpy as np

from ._native import C128, PREC, lib
from .device import DeviceTensor, to_host_mpo

__all__ = ["updateleft", "updateright"]


def _dtype(*ts):
    return np.complex128 if any(getattr(t, "code", 0) == C128 or
                                (isinstance(t, np.ndarray) and np.iscomplexobj(t))
                                for t in ts) else np.float64


def updateleft(hold, A, W, B, precision="fp64"):
    """hnew[b',w2,b] = sum hold[a',w,a] B[a,s,b] W[w,s',w2,s] conj(A[a',s',b'])
    (mpo/transfer.jl:31-34).  W=None is the operator-less update (:42-45)."""
    Dl, d, Dr = B.shape
    if A.shape != B.shape:
        raise ValueError("DimensionMismatch: A %s vs B %s" % (A.shape, B.shape))
    wl = hold.shape[1]
    wr = wl if W is None else W.shape[2]
    if hold.shape != (Dl, wl, Dl) or (W is not None and (W.shape[0] != wl or W.shape[1] != d)):
        raise ValueError("DimensionMismatch in updateleft")
    dt = _dtype(hold, A, B, W)
    hnew = DeviceTensor((Dr, wr, Dr), dt, hold.h)
    wbuf = None if W is None else to_host_mpo(W, dt)
    hold.h.check(lib().fmpt_updateleft(hold.h.ptr, hnew.code, PREC[precision], hold.ptr, A.ptr,
                                       None if wbuf is None else wbuf.ctypes.data, B.ptr,
                                       hnew.ptr, Dl, d, Dr, wl, wr))
    return hnew


def updateright(hold, A, W, B, precision="fp64"):
    """hnew[a',w,a] = sum hold[b',w2,b] B[a,s,b] W[w,s',w2,s] conj(A[a',s',b'])
    (mpo/transfer.jl:26-29).  W=None is the operator-less update (:37-40)."""
    Dl, d, Dr = B.shape
    if A.shape != B.shape:
        raise ValueError("DimensionMismatch: A %s vs B %s" % (A.shape, B.shape))
    wr = hold.shape[1]
    wl = wr if W is None else W.shape[0]
    if hold.shape != (Dr, wr, Dr) or (W is not None and (W.shape[2] != wr or W.shape[1] != d)):
        raise ValueError("DimensionMismatch in updateright")
    dt = _dtype(hold, A, B, W)
    hnew = DeviceTensor((Dl, wl, Dl), dt, hold.h)
    wbuf = None if W is None else to_host_mpo(W, dt)
    hold.h.check(lib().fmpt_updateright(hold.h.ptr, hnew.code, PREC[precision], hold.ptr, A.ptr,
                                        None if wbuf is None else wbuf.ctypes.data, B.ptr,
                                        hnew.ptr, Dl, d, Dr, wl, wr))
    return hnew
