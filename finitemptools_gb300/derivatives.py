"""Effective-Hamiltonian actions (algorithms/derivatives.jl) and the Krylov
solvers that apply them (auxiliary/simple_lanczos.jl, KrylovKit.exponentiate
as called from algorithms/tdvp.jl:3-6).

MPO tensors are host numpy arrays W[wl, s_out, wr, s_in]; states and
environments are DeviceTensors.  ``precision`` selects the arithmetic of
the contractions: "fp64" (plain form), "tf32x3", "tf32" or "bf16" (tensor
cores, FP32 accumulation).
"""

import ctypes

import numpy as np

from ._native import C128, PREC, lib
from .device import DeviceTensor, to_host_mpo

__all__ = ["ac_prime", "ac2_prime", "c_prime", "HeffOp", "simple_lanczos_solver",
           "exponentiate"]


def _prec(p):
    try:
        return PREC[p]
    except KeyError:
        raise ValueError("unknown precision %r" % (p,))


def _check_env(env, D, name):
    if env.shape[0] != D or env.shape[2] != D:
        raise ValueError("DimensionMismatch: %s has shape %s, bond %d" % (name, env.shape, D))


class HeffOp:
    """A prepared effective Hamiltonian (fmpt_op).  The environments it
    references must stay alive and unchanged while it is used."""

    def __init__(self, kind, hleft, hright, W1=None, W2=None, precision="fp64", dims=None,
                 dtype=None):
        self.h = hleft.h
        self.kind = kind
        self.hleft, self.hright = hleft, hright          # keep them alive
        cplx = (dtype is not None and np.dtype(dtype) == np.complex128) or \
            hleft.code == C128 or hright.code == C128 or \
            any(W is not None and np.iscomplexobj(W) for W in (W1, W2))
        self.dtype = np.complex128 if cplx else np.float64
        code = C128 if cplx else 0
        if hleft.code != code or hright.code != code:
            raise TypeError("environments must have the operator's dtype")
        self._bufs = []
        op = ctypes.c_void_p()
        Dl, wl = hleft.shape[0], hleft.shape[1]
        Dr, wr = hright.shape[0], hright.shape[1]
        _check_env(hleft, Dl, "hleft")
        _check_env(hright, Dr, "hright")
        if kind == "ac2":
            W1 = np.asarray(W1)
            W2 = np.asarray(W2)
            if W1.shape[0] != wl or W2.shape[2] != wr or W1.shape[2] != W2.shape[0]:
                raise ValueError("DimensionMismatch: MPO bonds vs environments")
            d1, d2, wm = W1.shape[1], W2.shape[1], W1.shape[2]
            b1, b2 = to_host_mpo(W1, self.dtype), to_host_mpo(W2, self.dtype)
            self._bufs = [b1, b2]
            self.shape = (Dl, d1, d2, Dr)
            self.h.check(lib().fmpt_op_ac2(self.h.ptr, code, _prec(precision), b1.ctypes.data,
                                           b2.ctypes.data, hleft.ptr, hright.ptr, Dl, d1, d2, Dr,
                                           wl, wm, wr, ctypes.byref(op)))
        elif kind == "ac":
            W1 = np.asarray(W1)
            if W1.shape[0] != wl or W1.shape[2] != wr:
                raise ValueError("DimensionMismatch: MPO bonds vs environments")
            d = W1.shape[1]
            b1 = to_host_mpo(W1, self.dtype)
            self._bufs = [b1]
            self.shape = (Dl, d, Dr)
            self.h.check(lib().fmpt_op_ac(self.h.ptr, code, _prec(precision), b1.ctypes.data,
                                          hleft.ptr, hright.ptr, Dl, d, Dr, wl, wr,
                                          ctypes.byref(op)))
        elif kind == "c":
            if wl != wr:
                raise ValueError("DimensionMismatch: c_prime needs equal MPO bonds")
            self.shape = (Dl, Dr)
            self.h.check(lib().fmpt_op_c(self.h.ptr, code, _prec(precision), hleft.ptr,
                                         hright.ptr, Dl, Dr, wl, ctypes.byref(op)))
        else:
            raise ValueError(kind)
        self.ptr = op

    def __del__(self):
        try:
            if self.ptr:
                lib().fmpt_op_destroy(self.ptr)
        except Exception:
            pass
        self.ptr = None

    def _check_x(self, x):
        if tuple(x.shape) != tuple(self.shape):
            raise ValueError("DimensionMismatch: x %s vs operator %s" % (x.shape, self.shape))
        if x.dtype != self.dtype:
            raise TypeError("x dtype %s vs operator %s" % (x.dtype, self.dtype))

    def __call__(self, x, out=None):
        self._check_x(x)
        y = out if out is not None else DeviceTensor(self.shape, self.dtype, self.h)
        self.h.check(lib().fmpt_op_apply(self.ptr, x.ptr, y.ptr))
        return y

    def set_projectors(self, projectors):
        """Compose the operator with _project! (dmrgexcited.jl:1-6): after every
        application y -= dot(y, p) p for each device tensor p in order."""
        for p in projectors:
            self._check_x(p)
        self._proj = list(projectors)                     # keep them alive
        arr = (ctypes.c_void_p * max(1, len(self._proj)))(*[p.ptr for p in self._proj])
        self.h.check(lib().fmpt_op_set_projectors(self.ptr, len(self._proj), arr))

    def lanczos(self, x0, kmax=10, btol=1e-8, reorth=False):
        """simple_lanczos_solver(f, x0, "SR", kmax, btol) -> (eval, evec, info, niter)."""
        self._check_x(x0)
        out = DeviceTensor(self.shape, self.dtype, self.h)
        ev = ctypes.c_double()
        info = ctypes.c_int()
        it = ctypes.c_int()
        self.h.check(lib().fmpt_lanczos_ground(self.ptr, x0.ptr, int(kmax), float(btol),
                                               1 if reorth else 0, ctypes.byref(ev), out.ptr,
                                               ctypes.byref(info), ctypes.byref(it)))
        return ev.value, out, info.value, it.value

    def eigsolve(self, x0, num=1, which="SR", krylovdim=30, maxiter=100, tol=1e-12):
        """eigsolve(f, x0, num, which, Lanczos()) (algorithms/exactdiag.jl:28): the
        num lowest ("SR") or highest ("LR") eigenpairs by thick-restart Lanczos.
        Returns (values, vectors, info) with info = {converged, residuals, applies}."""
        self._check_x(x0)
        if which not in ("SR", "SA", "LR", "LA"):
            raise ValueError("which must be 'SR' or 'LR'")
        num = int(num)
        per = DeviceTensor(self.shape, self.dtype, self.h).nbytes
        buf = DeviceTensor((per // 8 * num,), np.float64, self.h)
        vals = (ctypes.c_double * num)()
        res = (ctypes.c_double * num)()
        nconv, napply = ctypes.c_int(), ctypes.c_int()
        self.h.check(lib().fmpt_eigsolve(self.ptr, x0.ptr, num, int(krylovdim), int(maxiter),
                                         float(tol), 1 if which in ("LR", "LA") else 0, vals,
                                         buf.ptr, res, ctypes.byref(nconv), ctypes.byref(napply)))
        vecs = []
        for i in range(num):
            v = DeviceTensor(self.shape, self.dtype, self.h)
            self.h.check(lib().fmpt_memcpy_d2d(self.h.ptr, v.ptr, buf.ptr + i * per, per))
            vecs.append(v)
        info = {"converged": nconv.value, "residuals": list(res), "applies": napply.value}
        return list(vals), vecs, info

    def exponentiate(self, t, x, tol=1e-8, krylovdim=30):
        """exp(t * H) x (KrylovKit.exponentiate as used by _exp_evolve)."""
        self._check_x(x)
        t = complex(t)
        out = DeviceTensor(self.shape, self.dtype, self.h)
        info = ctypes.c_int()
        self.h.check(lib().fmpt_exponentiate(self.ptr, t.real, t.imag, x.ptr, out.ptr,
                                             int(krylovdim), float(tol), ctypes.byref(info)))
        return out


def ac_prime(x, m, hleft, hright, precision="fp64"):
    """derivatives.jl:2-4 (dense) -- one-site H_eff * x."""
    return HeffOp("ac", hleft, hright, W1=m, precision=precision, dtype=x.dtype)(x)


def ac2_prime(x, h1, h2, hleft, hright, precision="fp64"):
    """derivatives.jl:20-22 (dense) -- two-site H_eff * x."""
    return HeffOp("ac2", hleft, hright, W1=h1, W2=h2, precision=precision, dtype=x.dtype)(x)


def ac2_prime_host(x, h1, h2, hleft, hright, precision="fp64", handle=None):
    """derivatives.jl:20-22 on host arrays (fmpt_ac2_prime_host): numpy x [Dl,d1,d2,Dr],
    hleft [Dl,wl,Dl], hright [Dr,wr,Dr], MPO tensors [wl,d1',wm,d1] and [wm,d2',wr,d2];
    returns y as a numpy array.  Real data in a mixed precision pipelines the
    transfers with the compute."""
    from .device import default_handle, to_host_buffer
    h = handle or default_handle()
    x, hleft, hright = np.asarray(x), np.asarray(hleft), np.asarray(hright)
    W1, W2 = np.asarray(h1), np.asarray(h2)
    cplx = any(np.iscomplexobj(a) for a in (x, hleft, hright, W1, W2))
    dt = np.complex128 if cplx else np.float64
    Dl, d1, d2, Dr = x.shape
    wl, wm, wr = W1.shape[0], W1.shape[2], W2.shape[2]
    if hleft.shape != (Dl, wl, Dl) or hright.shape != (Dr, wr, Dr) or W2.shape[0] != wm:
        raise ValueError("DimensionMismatch in ac2_prime_host")
    # every host buffer stays referenced here until the call returns
    bufs = [to_host_buffer(a, dt) for a in (x, W1, W2, hleft, hright)]
    y = np.empty_like(bufs[0])
    h.check(lib().fmpt_ac2_prime_host(h.ptr, C128 if cplx else 0, _prec(precision),
                                      bufs[0].ctypes.data, bufs[1].ctypes.data,
                                      bufs[2].ctypes.data, bufs[3].ctypes.data,
                                      bufs[4].ctypes.data, y.ctypes.data, Dl, d1, d2, Dr, wl, wm,
                                      wr))
    n = x.size
    flat = y[:n] + 1j * y[n:] if cplx else y
    return flat.reshape(x.shape, order="F")


def c_prime(x, hleft, hright, precision="fp64"):
    """derivatives.jl:52-54 -- zero-site H_eff * C."""
    return HeffOp("c", hleft, hright, precision=precision, dtype=x.dtype)(x)


def simple_lanczos_solver(op, v, which="SR", kmax=10, btol=1.0e-8, reorth=False):
    """auxiliary/simple_lanczos.jl:83-120 on a prepared HeffOp."""
    if which not in ("SR", "SA"):
        raise ValueError("only the lowest eigenpair ('SR') is implemented")
    return op.lanczos(v, kmax, btol, reorth)


def exponentiate(op, t, x, tol=1e-8, krylovdim=30):
    return op.exponentiate(t, x, tol, krylovdim)
