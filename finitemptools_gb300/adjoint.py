"""Differentiable one-site TDVP: the discrete adjoint of TDVP1 on the device.

Gradient of an observable after a TDVP1 trajectory (algorithms/tdvp.jl:19-69)
with respect to the MPO site tensors, and from there to per-site couplings
(the transverse fields h_i of -sum Z Z - sum h_i X).  The reference has no
gradient code (ChainRulesCore is not one of its dependencies); this is the
reverse-mode counterpart of its TDVP1 sweep, built from GEMM-shaped adjoint
contractions on the device:

- ac_prime(b, W, L, R) paired with a: Lbar = conj(updateright(R, a, W, b)),
  Rbar = conj(updateleft(L, a, W, b)), Wbar = fmpt_wgrad(a, L, b, R);
- environment updates: the old environment's cotangent is the conjugated
  update from the other side, the bra/ket cotangents are ac_prime
  applications with L, W, R permuted (fmpt_swap13 for L^dagger and R^T);
- y = exp(t H) x: xbar = exp(conj(t) H) ybar, and the H-derivative by
  8-point Gauss-Legendre quadrature of <exp(s conj(t) H) ybar, dH exp((1-s) t H) x>
  over s, every node from one Krylov space per vector (fmpt_expm_nodes);
- QR / LQ gauge moves: fmpt_qr_adjoint (thin QR with real diag(R)).

Cotangents follow zbar = dL/dRe z + i dL/dIm z, so dL = Re sum conj(zbar) dz.
Checkpointing: only the MPS is stored every ``checkpoint`` steps; the
environments at a step boundary are exactly init_hstorage(mps, W) (the right
sweep rebuilds them with the same updates), so each block is recomputed from
its checkpoint, taped, and reversed, and its start-environment cotangents flow
back through that init chain.
"""

import ctypes

import numpy as np

from ._native import C128, lib
from .auxiliary import axpy, gemm, leftorth, rightorth, scal
from .derivatives import HeffOp, ac_prime
from .device import DeviceTensor
from .envs import _mpo_tensors, l_LL, r_RR
from .utilities import MPOHamiltonian
from .transfer import updateleft, updateright

__all__ = ["tdvp1_gradient", "tdvp1_forward", "tdvp1_backward", "tfi_field_gradient",
           "TDVP1Observable", "tdvp1_observable", "tfi_observable", "tfi_mpo_torch",
           "expm_nodes", "wgrad", "qr_adjoint", "gl_nodes"]


def gl_nodes(n=8):
    """Gauss-Legendre nodes and weights on [0, 1]."""
    s, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (s + 1.0), 0.5 * w


# ------------------------------------------------------------------ helpers
def _conj_(x):
    """In-place complex conjugate of a C128 device tensor (negate the imaginary plane)."""
    if x.code != C128:
        return x
    n = x.size
    c = (ctypes.c_double * 2)(-1.0, 0.0)
    x.h.check(lib().fmpt_scal(x.h.ptr, 0, n, c, x.ptr + 8 * n))
    return x


def _conj(x):
    return _conj_(x.copy())


def _swap13(x, conj=False):
    n0, n1, n2 = x.shape
    y = DeviceTensor((n2, n1, n0), x.dtype, x.h)
    x.h.check(lib().fmpt_swap13(x.h.ptr, x.code, x.ptr, y.ptr, n0, n1, n2, 1 if conj else 0))
    return y


def _acc(dst, src, a=1.0):
    """dst += a * src (dst None: a fresh copy)."""
    if src is None:
        return dst
    if dst is None:
        out = src.copy()
        if a != 1.0:
            scal(a, out)
        return out
    axpy(a, src, dst)
    return dst


def _mat(x, m, n):
    """The same device memory viewed as an m x n matrix (no copy)."""
    return x.view_as((m, n))


def expm_nodes(op, t, x, nodes, krylovdim=30):
    """[exp(s t H) x for s in nodes] from one Krylov space of x."""
    t = complex(t)
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    k = len(nodes)
    out = DeviceTensor((k,) + tuple(x.shape), x.dtype, x.h)
    err = ctypes.c_double()
    x.h.check(lib().fmpt_expm_nodes(op.ptr, t.real, t.imag, x.ptr, int(krylovdim), k,
                                    nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    out.ptr, ctypes.byref(err)))
    per = x.nbytes
    vecs = []
    for j in range(k):
        v = DeviceTensor(x.shape, x.dtype, x.h)
        x.h.check(lib().fmpt_memcpy_d2d(x.h.ptr, v.ptr, out.ptr + j * per, per))
        vecs.append(v)
    return vecs, err.value


def wgrad(a, Lenv, b, Renv):
    """conj(sum conj(a[a',s',b']) L[a',w,a] b[a,s,b] R[b',w2,b]) -> [w, s', w2, s]."""
    Dl, d, Dr = b.shape
    wl, wr = Lenv.shape[1], Renv.shape[1]
    out = DeviceTensor((wl, d, wr, d), np.complex128, a.h)
    a.h.check(lib().fmpt_wgrad(a.h.ptr, C128, a.ptr, Lenv.ptr, b.ptr, Renv.ptr, out.ptr,
                               Dl, d, Dr, wl, wr))
    return out


def qr_adjoint(Q, R, Qbar, Rbar, m, n):
    """Mbar (m x n) of the thin QR M = Q R (m >= n)."""
    Mb = DeviceTensor((m, n), np.complex128, Q.h)
    Q.h.check(lib().fmpt_qr_adjoint(Q.h.ptr, C128, Q.ptr, R.ptr, Qbar.ptr, Rbar.ptr, Mb.ptr,
                                    m, n))
    return Mb


def _conj_transpose(M):
    """M^H of an m x n device matrix."""
    m, n = M.shape
    y = _swap13(M.view_as((m, 1, n)), conj=True)
    M.view_as((m, n))
    return y.view_as((n, m))


# -------------------------------------------------------- primitive adjoints
def _ac_adjoint(a, b, W, Le, Re):
    Lb = _conj_(updateright(Re, a, W, b))
    Rb = _conj_(updateleft(Le, a, W, b))
    return Lb, wgrad(a, Le, b, Re), Rb


def _c_adjoint(a, C, Le, Re):
    Dl, Dr = C.shape
    a3 = a.copy().view_as((Dl, 1, Dr))
    c3 = C.copy().view_as((Dl, 1, Dr))
    Lb = _conj_(updateright(Re, a3, None, c3))
    Rb = _conj_(updateleft(Le, a3, None, c3))
    return Lb, Rb


def _expo_backward(run, kind, t, x, ybar, W, Le, Re, nodes):
    """Cotangents (xbar, Lbar, Wbar, Rbar) of y = exp(t H) x (H Hermitian).  The
    exponentials run in the run's arithmetic; the contractions that pair the
    quadrature vectors stay FP64."""
    krylovdim = run.krylovdim
    op = run.op(kind, Le, Re, W)
    s, w = nodes
    bs, _ = expm_nodes(op, t, x, 1.0 - s, krylovdim)
    as_, _ = expm_nodes(op, np.conj(t), ybar, np.concatenate([s, [1.0]]), krylovdim)
    xbar = as_[-1]
    Lb = Rb = Wb = None
    for k in range(len(s)):
        ak = scal(np.conj(t), as_[k])
        if kind == "ac":
            l, wg, r = _ac_adjoint(ak, bs[k], W, Le, Re)
            Wb = _acc(Wb, wg, w[k])
        else:
            l, r = _c_adjoint(ak, bs[k], Le, Re)
        Lb = _acc(Lb, l, w[k])
        Rb = _acc(Rb, r, w[k])
    return xbar, Lb, Wb, Rb


def _updateleft_backward(hbar, hold, A, W, B):
    """(holdbar, Abar, Wbar, Bbar) of hnew = updateleft(hold, A, W, B)."""
    hc = _conj(hbar)
    hb_old = _conj_(updateright(hc, A, W, B))
    Ab = ac_prime(B, W, hold, hc)
    Wsw = np.conj(np.transpose(W, (0, 3, 2, 1)))
    Bb = ac_prime(A, Wsw, _swap13(hold, conj=True), _swap13(hbar))
    Wb = wgrad(A, hold, B, hc)
    return hb_old, Ab, Wb, Bb


def _updateright_backward(hbar, hold, A, W, B):
    """(holdbar, Abar, Wbar, Bbar) of hnew = updateright(hold, A, W, B)."""
    hc = _conj(hbar)
    hb_old = _conj_(updateleft(hc, A, W, B))
    Ab = ac_prime(B, W, hc, hold)
    Wsw = np.conj(np.transpose(W, (0, 3, 2, 1)))
    Bb = ac_prime(A, Wsw, _swap13(hbar), _swap13(hold, conj=True))
    Wb = wgrad(A, hc, B, hold)
    return hb_old, Ab, Wb, Bb


def _qr_backward(Q3, R, Qb3, Rb):
    Dl, d, k = Q3.shape
    Qm = Q3.copy().view_as((Dl * d, k))
    Qbm = Qb3.copy().view_as((Dl * d, k))
    return qr_adjoint(Qm, R, Qbm, Rb, Dl * d, k).view_as((Dl, d, k))


def _lq_backward(Lm, Q3, Lb, Qb3):
    """Mbar of M = L Q computed as M^H = Q' R' (fmpt_lq): Q' = Q^H, R' = L^H."""
    r, d, Dr = Q3.shape
    Qp = _conj_transpose(Q3.copy().view_as((r, d * Dr)))      # (d Dr) x r
    Rp = _conj_transpose(Lm.copy())                            # r x m  (m = r here)
    Qpb = _conj_transpose(Qb3.copy().view_as((r, d * Dr)))
    Rpb = _conj_transpose(Lb.copy())
    Nb = qr_adjoint(Qp, Rp, Qpb, Rpb, d * Dr, r)
    return _conj_transpose(Nb).view_as((Lm.shape[0], d, Dr))


# -------------------------------------------------------------- TDVP1 tape
class _Run:
    def __init__(self, Ws, dt, exptol, krylovdim, precision="fp64"):
        self.Ws = Ws
        self.dt = dt
        self.exptol = exptol
        self.krylovdim = krylovdim
        self.precision = precision

    def op(self, kind, Le, Re, W=None):
        """H_eff of one site ("ac", MPO tensor W) or one bond ("c") in the run's
        arithmetic.  The tensor-core forms embed complex states as real GEMMs and
        need a real MPO, so a real-valued W is handed over as real."""
        if kind != "ac":
            W = None
        elif self.precision != "fp64" and not np.any(np.imag(W)):
            W = np.ascontiguousarray(np.real(W))
        return HeffOp(kind, Le, Re, W1=W, precision=self.precision, dtype=np.complex128)


def _init_envs(run, mps, tape=None):
    """init_hstorage! (finiteenv.jl:1-21): right environments of every site."""
    L = len(mps)
    Ws = run.Ws
    h = mps[0].h
    hs = [None] * (L + 1)
    hs[0] = l_LL(Ws[0].shape[0], np.complex128, h, True)
    hs[L] = r_RR(Ws[-1].shape[2], np.complex128, h, True)
    for i in range(L - 1, 0, -1):
        if tape is not None:
            tape.append((i, hs[i + 1], mps[i]))
        hs[i] = updateright(hs[i + 1], mps[i], Ws[i], mps[i])
    return hs


def _step(run, mps, hs, rec=None):
    """One TDVP1 sweep (tdvp.jl:19-69), the same device calls as the product's
    TDVP1 driver; rec (a list) receives one record per site update."""
    Ws, dt, L = run.Ws, run.dt, len(mps)
    tol2, tol1 = run.exptol / abs(dt / 2), run.exptol / abs(dt)
    for s in range(L - 1):
        x = mps[s]
        op = run.op("ac", hs[s], hs[s + 1], Ws[s])
        tmp = op.exponentiate(dt / 2, x, tol2, run.krylovdim)
        del op
        Dl, d, Dr = x.shape
        Q, R = leftorth(tmp, Dl * d, Dr)
        k = Q.shape[1]
        Q3 = Q.view_as((Dl, d, k))
        hnew = updateleft(hs[s], Q3, Ws[s], Q3)
        opc = run.op("c", hnew, hs[s + 1])
        v = opc.exponentiate(-dt / 2, R, tol2, run.krylovdim)
        del opc
        B = mps[s + 1]
        if rec is not None:
            rec.append({"kind": "left", "s": s, "x": x, "Le": hs[s], "Re": hs[s + 1], "Q": Q3,
                        "R": R, "hnew": hnew, "v": v, "B": B})
        mps[s] = Q3
        mps[s + 1] = gemm(v, B, (k, B.shape[1], B.shape[2]), k, B.shape[1] * B.shape[2], Dr)
        hs[s + 1] = hnew
    s = L - 1
    x = mps[s]
    if rec is not None:
        rec.append({"kind": "last", "s": s, "x": x, "Le": hs[s], "Re": hs[s + 1]})
    op = run.op("ac", hs[s], hs[s + 1], Ws[s])
    mps[s] = op.exponentiate(dt, x, tol1, run.krylovdim)
    del op
    for s in range(L - 2, -1, -1):
        Bt = mps[s + 1]
        Dl, d, Dr = Bt.shape
        Lm, Q = rightorth(Bt, Dl, d * Dr)
        r = Q.shape[0]
        Q3 = Q.view_as((r, d, Dr))
        hold = hs[s + 2]
        hnew = updateright(hold, Q3, Ws[s + 1], Q3)
        Lc = hs[s + 1]
        opc = run.op("c", Lc, hnew)
        v = opc.exponentiate(-dt / 2, Lm, tol2, run.krylovdim)
        del opc
        A = mps[s]
        Av = gemm(A, v, (A.shape[0], A.shape[1], r), A.shape[0] * A.shape[1], r, Dl)
        if rec is not None:
            rec.append({"kind": "right", "s": s, "Lm": Lm, "Q": Q3, "hold": hold, "Lc": Lc,
                        "Le": hs[s], "hnew": hnew, "v": v, "A": A, "Av": Av})
        mps[s + 1] = Q3
        hs[s + 1] = hnew
        op = run.op("ac", hs[s], hnew, Ws[s])
        mps[s] = op.exponentiate(dt / 2, Av, tol2, run.krylovdim)
        del op


def _observable(mps, site, Op, keep=False):
    """(n1, n0) = (<psi|O_site|psi>, <psi|psi>) by right-to-left chains (0-based site)."""
    L = len(mps)
    h = mps[0].h
    d = mps[0].shape[1]
    I = np.eye(d, dtype=np.complex128).reshape(1, d, 1, d)
    O = np.asarray(Op, dtype=np.complex128).reshape(1, d, 1, d)
    one = np.ones((1, 1, 1), dtype=np.complex128)
    h1 = {L: DeviceTensor.from_numpy(one, h, np.complex128)}
    h0 = {L: DeviceTensor.from_numpy(one, h, np.complex128)}
    for i in range(L - 1, -1, -1):
        h1[i] = updateright(h1[i + 1], mps[i], O if i == site else I, mps[i])
        h0[i] = updateright(h0[i + 1], mps[i], I, mps[i])
    n1 = complex(h1[0].numpy().reshape(-1)[0])
    n0 = complex(h0[0].numpy().reshape(-1)[0])
    return (n1, n0, h1, h0, O, I) if keep else (n1, n0)


def _observable_backward(mps, site, Op):
    n1, n0, h1, h0, O, I = _observable(mps, site, Op, keep=True)
    h = mps[0].h
    b1 = DeviceTensor.from_numpy(np.full((1, 1, 1), np.conj(1.0 / n0)), h, np.complex128)
    b0 = DeviceTensor.from_numpy(np.full((1, 1, 1), np.conj(-n1 / n0 ** 2)), h, np.complex128)
    grads = []
    for i in range(len(mps)):
        hb1, Ab1, _, Bb1 = _updateright_backward(b1, h1[i + 1], mps[i], O if i == site else I,
                                                 mps[i])
        hb0, Ab0, _, Bb0 = _updateright_backward(b0, h0[i + 1], mps[i], I, mps[i])
        g = Ab1
        for t in (Bb1, Ab0, Bb0):
            axpy(1.0, t, g)
        grads.append(g)
        b1, b0 = hb1, hb0
    return float(np.real(n1 / n0)), grads


def _reverse_block(run, rec, init_tape, mb, Wb, nodes):
    """Reverse one recomputed block: mb (site cotangents at the block end) ->
    cotangents at the block start; Wbar accumulated into Wb."""
    Ws, dt = run.Ws, run.dt
    L = len(Ws)
    hb = [None] * (L + 1)

    def add(i, g):
        hb[i] = _acc(hb[i], g)

    def pop(i):
        g = hb[i]
        hb[i] = None
        return g

    for r in reversed(rec):
        s = r["s"]
        if r["kind"] == "right":
            xb, lb, wb, rb = _expo_backward(run, "ac", dt / 2, r["Av"], mb[s], Ws[s], r["Le"],
                                            r["hnew"], nodes)
            Wb[s] = _acc(Wb[s], wb)
            add(s, lb)
            add(s + 1, rb)
            A, v = r["A"], r["v"]
            Dl, d, k = A.shape
            rr = v.shape[1]
            Cm = xb.view_as((Dl * d, rr))
            mb[s] = gemm(Cm, v, (Dl, d, k), Dl * d, k, rr, tb="C")             # Avbar v^H
            vb = gemm(A, Cm, (k, rr), k, rr, Dl * d, ta="C", lda=Dl * d)      # A^H Avbar
            hnb = pop(s + 1)
            Lmb, lb2, _, rb2 = _expo_backward(run, "c", -dt / 2, r["Lm"], vb, None, r["Lc"],
                                              r["hnew"], nodes)
            add(s + 1, lb2)
            hnb = _acc(hnb, rb2)
            W1 = Ws[s + 1]
            hold_b, Ab, wb, Bb = _updateright_backward(hnb, r["hold"], r["Q"], W1, r["Q"])
            add(s + 2, hold_b)
            Wb[s + 1] = _acc(Wb[s + 1], wb)
            Qb = Ab
            axpy(1.0, Bb, Qb)
            if mb[s + 1] is not None:
                axpy(1.0, mb[s + 1], Qb)
            mb[s + 1] = _lq_backward(r["Lm"], r["Q"], Lmb, Qb)
        elif r["kind"] == "last":
            xb, lb, wb, rb = _expo_backward(run, "ac", dt, r["x"], mb[s], Ws[s], r["Le"],
                                            r["Re"], nodes)
            mb[s] = xb
            Wb[s] = _acc(Wb[s], wb)
            add(s, lb)
            add(s + 1, rb)
        else:
            hnb = pop(s + 1)
            B, v = r["B"], r["v"]
            k, Dlb = v.shape
            Cm = mb[s + 1].view_as((k, B.shape[1] * B.shape[2]))
            vb = gemm(Cm, B, (k, Dlb), k, Dlb, B.shape[1] * B.shape[2], tb="C", ldb=Dlb)
            mb[s + 1] = gemm(v, Cm, B.shape, Dlb, B.shape[1] * B.shape[2], k, ta="C")
            Qb = mb[s]
            mb[s] = None
            Rb, lb, _, rb = _expo_backward(run, "c", -dt / 2, r["R"], vb, None, r["hnew"],
                                           r["Re"], nodes)
            hnb = _acc(hnb, lb)
            add(s + 1, rb)
            hold_b, Ab, wb, Bb = _updateleft_backward(hnb, r["Le"], r["Q"], Ws[s], r["Q"])
            add(s, hold_b)
            Wb[s] = _acc(Wb[s], wb)
            axpy(1.0, Ab, Qb)
            axpy(1.0, Bb, Qb)
            tmpb = _qr_backward(r["Q"], r["R"], Qb, Rb)
            xb, lb, wb, rb = _expo_backward(run, "ac", dt / 2, r["x"], tmpb, Ws[s], r["Le"],
                                            r["Re"], nodes)
            mb[s] = xb
            Wb[s] = _acc(Wb[s], wb)
            add(s, lb)
            add(s + 1, rb)
    # the block's start environments are init_hstorage(mps_start, W)
    for i, hnext, A in reversed(init_tape):
        g = pop(i)
        if g is None:
            continue
        hold_b, Ab, wb, Bb = _updateright_backward(g, hnext, A, Ws[i], A)
        add(i + 1, hold_b)
        Wb[i] = _acc(Wb[i], wb)
        mb[i] = _acc(mb[i], Ab)
        axpy(1.0, Bb, mb[i])
    return mb


class TDVP1Tape:
    """What the reverse pass of a TDVP1 trajectory needs: the run (MPO tensors,
    step, tolerances, arithmetic), the MPS every ``checkpoint`` steps and the
    final state.  Held by TDVP1Observable between forward and backward."""

    def __init__(self, run, checkpoints, nsteps, final_mps, site, Op):
        self.run, self.checkpoints, self.nsteps = run, checkpoints, nsteps
        self.final_mps, self.site, self.Op = final_mps, site, Op


def tdvp1_forward(mpo, psi0, stepsize, nsteps, site, Op, checkpoint=10, exptol=1e-12,
                  krylovdim=30, precision="fp64"):
    """Re <Op_site>(T) (``site`` 1-based) after ``nsteps`` TDVP1 sweeps of size
    ``stepsize`` (real time: -1j*dt) from psi0 (a complex FiniteMPS, not
    modified), and the tape for tdvp1_backward.  ``mpo`` is an MPOHamiltonian or
    a list of dense site tensors W[wl, s_out, wr, s_in]: bulk Schur grids (the
    environments close them with the boundary vectors l_LL / r_RR) or a strict
    FiniteMPO (first and last MPO bonds 1, where those vectors are [1]).  ``precision`` is the
    arithmetic of the Krylov exponentials (forward and adjoint); "fp64" is the
    reference's, the tensor-core forms ("tf32x3", ...) need a real MPO."""
    if checkpoint < 1:
        raise ValueError("checkpoint must be >= 1")
    L = len(psi0)
    if isinstance(mpo, MPOHamiltonian):
        Ws, _ = _mpo_tensors(mpo, L)
    else:
        Ws = list(mpo)
        if len(Ws) != L:
            raise ValueError("DimensionMismatch: MPO length %d vs MPS length %d" % (len(Ws), L))
    Ws = [np.asarray(W, dtype=np.complex128) for W in Ws]
    run = _Run(Ws, complex(stepsize), exptol, krylovdim, precision)
    mps = [psi0[i].copy() for i in range(1, L + 1)]
    checkpoints = []
    hs = _init_envs(run, mps)
    for step in range(nsteps):
        if step % checkpoint == 0:
            checkpoints.append((step, [A.copy() for A in mps]))
        _step(run, mps, hs)
    del hs
    n1, n0 = _observable(mps, site - 1, Op)
    return float(np.real(n1 / n0)), TDVP1Tape(run, checkpoints, nsteps, mps, site, Op)


def tdvp1_backward(tape, quad_nodes=8):
    """Gradient of tdvp1_forward's value with respect to every MPO site tensor
    (numpy arrays, zbar = dL/dRe W + i dL/dIm W).  Each checkpoint block is
    recomputed from its MPS, taped and reversed, last block first."""
    run = tape.run
    L = len(run.Ws)
    nodes = gl_nodes(quad_nodes)
    _, mb = _observable_backward(tape.final_mps, tape.site - 1, tape.Op)
    Wb = [None] * L
    cps = tape.checkpoints
    for k in range(len(cps) - 1, -1, -1):
        start, snap = cps[k]
        stop = cps[k + 1][0] if k + 1 < len(cps) else tape.nsteps
        mps = [A.copy() for A in snap]
        init_tape = []
        hs = _init_envs(run, mps, init_tape)
        rec = []
        for _ in range(start, stop):
            _step(run, mps, hs, rec)
        mb = _reverse_block(run, rec, init_tape, mb, Wb, nodes)
        del rec, init_tape, hs
    return [np.zeros(W.shape, dtype=np.complex128) if g is None else g.numpy() for W, g in
            zip(run.Ws, Wb)]


def tdvp1_gradient(mpo, psi0, stepsize, nsteps, site, Op, checkpoint=10, exptol=1e-12,
                   krylovdim=30, quad_nodes=8, precision="fp64"):
    """Value and MPO-tensor gradient of Re <Op_site>(T) (``site`` 1-based) after
    ``nsteps`` TDVP1 sweeps of size ``stepsize`` (real time: -1j*dt) from psi0
    (a complex FiniteMPS, not modified).  Returns (value, [Wbar_i] as numpy
    arrays, one per site).  Only every ``checkpoint``-th MPS is kept; each
    block is recomputed and reversed in turn."""
    value, tape = tdvp1_forward(mpo, psi0, stepsize, nsteps, site, Op, checkpoint, exptol,
                                krylovdim, precision)
    return value, tdvp1_backward(tape, quad_nodes)


def _field_grad(Wb):
    """dL/dh_i from the site-tensor cotangents of the TFI MPO (utilities.tfi_mpo):
    W[0, :, 2, :] = -h X, so dL/dh = Re sum conj(Wbar[0, :, 2, :]) * (-X)."""
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    return np.array([np.real(np.sum(np.conj(g[0, :, 2, :]) * (-X))) for g in Wb])


def tfi_field_gradient(h_fields, psi0, stepsize, nsteps, site, Op=None, **kw):
    """Re <Z_site>(T) and its gradient with respect to the transverse fields h_i
    of H = -sum Z_i Z_{i+1} - sum h_i X_i (utilities.tfi_mpo)."""
    from .utilities import tfi_mpo
    Op = np.diag([-1.0, 1.0]) if Op is None else Op
    value, Wb = tdvp1_gradient(tfi_mpo(h_fields), psi0, stepsize, nsteps, site, Op, **kw)
    return value, _field_grad(Wb)


# ------------------------------------------------------------ autograd boundary
def _torch():
    import torch
    return torch


def _make_function():
    torch = _torch()

    class TDVP1Observable(torch.autograd.Function):
        """Re <Op_site>(T) after a TDVP1 trajectory as a differentiable function of
        the MPO site tensors (complex128 torch tensors W[wl, s_out, wr, s_in], one
        per site).  forward runs the trajectory on the device and keeps only the
        checkpoints; backward runs the reverse pass (tdvp1_backward) and returns
        g * Wbar per site, Wbar = dL/dRe W + i dL/dIm W (torch's convention for a
        real loss of complex leaves).  The counterpart of a ChainRulesCore rrule
        around the reference's TDVP1 sweeps (algorithms/tdvp.jl:19-69)."""

        @staticmethod
        def forward(ctx, psi0, stepsize, nsteps, site, Op, opts, *Ws):
            mpo = [W.detach().cpu().numpy().astype(np.complex128) for W in Ws]
            value, tape = tdvp1_forward(mpo, psi0, stepsize, nsteps, site, Op,
                                        opts.get("checkpoint", 10), opts.get("exptol", 1e-12),
                                        opts.get("krylovdim", 30),
                                        opts.get("precision", "fp64"))
            ctx.tape = tape
            ctx.quad_nodes = opts.get("quad_nodes", 8)
            ctx.devices = [W.device for W in Ws]
            return torch.tensor(value, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            Wb = tdvp1_backward(ctx.tape, ctx.quad_nodes)
            ctx.tape = None
            grads = tuple(g.to(dev) * torch.from_numpy(w).to(dev)
                          for w, dev in zip(Wb, ctx.devices))
            return (None,) * 6 + grads

    return TDVP1Observable


_FUNCTION = None


def TDVP1Observable():
    """The torch.autograd.Function class (built on first use, so that importing
    this module does not import torch)."""
    global _FUNCTION
    if _FUNCTION is None:
        _FUNCTION = _make_function()
    return _FUNCTION


def tdvp1_observable(Ws, psi0, stepsize, nsteps, site, Op, **opts):
    """Differentiable Re <Op_site>(T): ``Ws`` a list of complex torch tensors
    (MPO site tensors, requires_grad as wanted).  Options: checkpoint, exptol,
    krylovdim, quad_nodes, precision."""
    return TDVP1Observable().apply(psi0, stepsize, nsteps, site, Op, dict(opts), *Ws)


def tfi_mpo_torch(h):
    """The TFI site tensors of utilities.tfi_mpo (w=3 Schur grid of
    -sum Z Z - sum h_i X, boundary vectors applied by the environments) as
    W_i = W(h=0) + h_i * dW/dh, built with torch ops from a real tensor of
    fields so that autograd carries dL/dW back to dL/dh."""
    torch = _torch()
    from .utilities import tfi_mpo
    w0 = np.asarray(tfi_mpo([0.0]).site_tensors(1)[0], dtype=np.complex128)
    w1 = np.asarray(tfi_mpo([1.0]).site_tensors(1)[0], dtype=np.complex128)
    base = torch.from_numpy(w0).to(h.device)
    field = torch.from_numpy(w1 - w0).to(h.device)
    hc = h.to(torch.complex128)
    return [base + hc[i] * field for i in range(h.shape[0])]


def tfi_observable(h, psi0, stepsize, nsteps, site, Op=None, **opts):
    """Differentiable Re <Op_site>(T) (default Op = Z) of the TFI chain with
    fields ``h`` (a real torch tensor): loss.backward() fills h.grad."""
    Op = np.diag([-1.0, 1.0]) if Op is None else Op
    return tdvp1_observable(tfi_mpo_torch(h), psi0, stepsize, nsteps, site, Op, **opts)
