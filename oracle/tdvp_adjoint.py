"""Discrete adjoint of one-site TDVP (test infrastructure only: the product
never imports this module).

The forward map is the reference's TDVP1 sweep (algorithms/tdvp.jl:19-69,
restated in oracle.algorithms.tdvp1_sweep) with every Krylov exponential taken
exactly (dense expm of the small effective Hamiltonian), so that the adjoint
below is the exact derivative of the forward map it differentiates.  The
reference has no gradient (ChainRulesCore is not a dependency), so this module
is pinned only by central finite differences of the same forward map.

Conventions.  A real loss L of complex tensors; the cotangent of z is
zbar = dL/dRe(z) + i dL/dIm(z), so that dL = Re sum(conj(zbar) * dz).
Index order as in oracle.core: A[a,s,b], W[wl,s',wr,s], L[a',w,a], R[b',w,b].

Building blocks (each derived from its forward contraction):
- ac_prime(b, W, L, R) paired with a:  Lbar = conj(updateright(R, a, W, b)),
  Rbar = conj(updateleft(L, a, W, b)), Wbar = conj(sum conj(a) L b R).
- y = exp(t H) x with H Hermitian:  xbar = exp(conj(t) H) ybar and the
  H-derivative  int_0^1 <exp(s conj(t) H) ybar, t dH exp((1-s) t H) x> ds,
  by Gauss-Legendre quadrature on s.
- thin QR M = Q R with real diag(R) (LAPACK):  Mbar = (I - Q Q^H) Qbar R^-H
  + Q Y R^-H + Q Rbar with K = Qbar^H Q - R Rbar^H, Y lower triangular,
  Y_ij = conj(K_ji) - K_ij (i > j), Y_ii = -i Im K_ii.
"""

import numpy as np
import scipy.linalg

from .core import ac_prime, c_prime, updateleft, updateright, l_LL_schur, r_RR_schur

__all__ = ["ac_adjoint", "c_adjoint", "expo_forward", "expo_backward", "qr_backward",
           "lq_forward", "lq_backward", "qr_forward", "updateleft_backward",
           "updateright_backward", "tdvp1_forward", "tdvp1_backward", "observable",
           "loss_and_grad", "fd_grad", "tfi_site_tensor"]

GL_NODES = 8


def tfi_site_tensor(hi):
    """Dense Schur grid (w=3) of -Z Z - h X at one site (the product's tfi_mpo)."""
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    Z = np.array([[-1.0, 0.0], [0.0, 1.0]])
    W = np.zeros((3, 2, 3, 2))
    W[0, :, 0, :] = np.eye(2)
    W[0, :, 1, :] = -Z
    W[0, :, 2, :] = -hi * X
    W[1, :, 2, :] = Z
    W[2, :, 2, :] = np.eye(2)
    return W


def dW_dh():
    """dW/dh_i of tfi_site_tensor (the -h X entry)."""
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    G = np.zeros((3, 2, 3, 2))
    G[0, :, 2, :] = -X
    return G


# ------------------------------------------------------------- contractions
def wgrad(a, L, b, R):
    """conj(sum conj(a[a',s',b']) L[a',w,a] b[a,s,b] R[b',w2,b]) -> [w,s',w2,s]."""
    G = np.einsum("pqr,pwa,asb,rxb->wqxs", np.conj(a), L, b, R)
    return np.conj(G)


def ac_adjoint(a, b, W, L, R):
    """(Lbar, Wbar, Rbar) of Re<a, ac_prime(b, W, L, R)>."""
    Lb = np.conj(updateright(R, a, W, b))
    Rb = np.conj(updateleft(L, a, W, b))
    return Lb, wgrad(a, L, b, R), Rb


def c_adjoint(a, C, L, R):
    """(Lbar, Rbar) of Re<a, c_prime(C, L, R)> (c_prime = sum_w L_w C R_w^T)."""
    w = L.shape[1]
    I = np.eye(w).reshape(w, 1, w, 1)
    a3 = a.reshape(a.shape[0], 1, a.shape[1])
    c3 = C.reshape(C.shape[0], 1, C.shape[1])
    Lb = np.conj(updateright(R, a3, I, c3))
    Rb = np.conj(updateleft(L, a3, I, c3))
    return Lb, Rb


def _heff(kind, W, L, R, shape):
    n = int(np.prod(shape))
    H = np.zeros((n, n), dtype=np.complex128)
    for j in range(n):
        e = np.zeros(n, dtype=np.complex128)
        e[j] = 1.0
        x = e.reshape(shape, order="F")
        y = ac_prime(x, W, L, R) if kind == "ac" else c_prime(x, L, R)
        H[:, j] = y.ravel(order="F")
    return H


def expo_forward(kind, t, x, W, L, R):
    """exp(t H_eff) x exactly (dense expm); H_eff = ac_prime or c_prime."""
    H = _heff(kind, W, L, R, x.shape)
    return (scipy.linalg.expm(t * H) @ x.ravel(order="F")).reshape(x.shape, order="F")


def expo_backward(kind, t, x, ybar, W, L, R, nodes=GL_NODES):
    """Cotangents (xbar, Lbar, Wbar, Rbar) of y = exp(t H(W, L, R)) x."""
    shape = x.shape
    H = _heff(kind, W, L, R, shape)
    xv = x.ravel(order="F")
    yb = ybar.ravel(order="F")
    xbar = (scipy.linalg.expm(np.conj(t) * H) @ yb).reshape(shape, order="F")
    s, wts = np.polynomial.legendre.leggauss(nodes)
    s = 0.5 * (s + 1.0)
    wts = 0.5 * wts
    Lb = np.zeros_like(L, dtype=np.complex128)
    Rb = np.zeros_like(R, dtype=np.complex128)
    Wb = np.zeros(W.shape, dtype=np.complex128) if W is not None else None
    for sk, wk in zip(s, wts):
        a = np.conj(t) * (scipy.linalg.expm(sk * np.conj(t) * H) @ yb)
        b = scipy.linalg.expm((1.0 - sk) * t * H) @ xv
        a = a.reshape(shape, order="F")
        b = b.reshape(shape, order="F")
        if kind == "ac":
            l, w, r = ac_adjoint(a, b, W, L, R)
            Wb += wk * w
        else:
            l, r = c_adjoint(a, b, L, R)
        Lb += wk * l
        Rb += wk * r
    return xbar, Lb, Wb, Rb


def qr_forward(A):
    """leftorth!(A, QR()) on A[a,s,b] as (a s) x b (LAPACK thin QR)."""
    Dl, d, Dr = A.shape
    Q, R = np.linalg.qr(A.reshape(Dl * d, Dr, order="F"), mode="reduced")
    return Q.reshape(Dl, d, Q.shape[1], order="F"), R


def qr_backward(Q, R, Qbar, Rbar):
    """Mbar of the thin QR M = Q R (real diagonal of R)."""
    K = Qbar.conj().T @ Q - R @ Rbar.conj().T
    Y = np.tril(K.conj().T - K, -1) + np.diag(-1j * np.imag(np.diag(K)))
    Rinv_h = np.linalg.inv(R).conj().T
    proj = Qbar - Q @ (Q.conj().T @ Qbar)
    return proj @ Rinv_h + Q @ Y @ Rinv_h + Q @ Rbar


def lq_forward(A):
    """rightorth(A, LQ()) on A[a,s,b] as a x (s b): M^T = Q R, L = R^T, Q' = Q^T."""
    Dl, d, Dr = A.shape
    M = A.reshape(Dl, d * Dr, order="F")
    Q, R = np.linalg.qr(M.T, mode="reduced")
    return R.T, Q.T.reshape(Q.shape[1], d, Dr, order="F"), (Q, R)


def lq_backward(qr_pair, Lbar, Qpbar):
    """Mbar of the LQ above from the cotangents of L (= R^T) and Q' (= Q^T)."""
    Q, R = qr_pair
    k = Q.shape[1]
    Qbar = Qpbar.reshape(k, -1, order="F").T
    Rbar = Lbar.T
    return qr_backward(Q, R, Qbar, Rbar).T


def updateleft_backward(hbar, hold, A, W, B):
    """(holdbar, Abar (bra), Wbar, Bbar (ket)) of hnew = updateleft(hold, A, W, B)."""
    hb_old = np.conj(updateright(np.conj(hbar), A, W, B))
    Ab = ac_prime(B, W, hold, np.conj(hbar))
    Wsw = np.conj(np.transpose(W, (0, 3, 2, 1)))
    Bb = ac_prime(A, Wsw, np.conj(np.transpose(hold, (2, 1, 0))), np.transpose(hbar, (2, 1, 0)))
    Wb = np.conj(np.einsum("rxb,pwa,asb,pqr->wqxs", np.conj(hbar), hold, B, np.conj(A)))
    return hb_old, Ab, Wb, Bb


def updateright_backward(hbar, hold, A, W, B):
    """(holdbar, Abar (bra), Wbar, Bbar (ket)) of hnew = updateright(hold, A, W, B)."""
    hb_old = np.conj(updateleft(np.conj(hbar), A, W, B))
    Ab = ac_prime(B, W, np.conj(hbar), hold)
    Wsw = np.conj(np.transpose(W, (0, 3, 2, 1)))
    Bb = ac_prime(A, Wsw, np.transpose(hbar, (2, 1, 0)), np.conj(np.transpose(hold, (2, 1, 0))))
    Wb = np.conj(np.einsum("pwa,rxb,asb,pqr->wqxs", np.conj(hbar), hold, B, np.conj(A)))
    return hb_old, Ab, Wb, Bb


# --------------------------------------------------------------- TDVP1 tape
def tdvp1_forward(Ws, mps0, dt, nsteps):
    """nsteps TDVP1 sweeps (tdvp.jl:19-69) from mps0 (exact exponentials).
    Returns the final MPS and a tape with one record per site update."""
    L = len(mps0)
    mps = [A.astype(np.complex128) for A in mps0]
    hs = [None] * (L + 1)
    hs[0] = l_LL_schur(Ws[0].shape[0], np.complex128)
    hs[L] = r_RR_schur(Ws[-1].shape[2], np.complex128)
    init = []
    for i in range(L - 1, 0, -1):               # init_hstorage! (finiteenv.jl:1-21)
        init.append((i, hs[i + 1], mps[i]))
        hs[i] = updateright(hs[i + 1], mps[i], Ws[i], mps[i])
    tape = []
    for _ in range(nsteps):
        for s in range(L - 1):                  # _leftsweep! (tdvp.jl:28-40)
            r = {"kind": "left", "s": s, "x": mps[s], "Le": hs[s], "Re": hs[s + 1],
                 "B": mps[s + 1]}
            tmp = expo_forward("ac", dt / 2, mps[s], Ws[s], hs[s], hs[s + 1])
            Q, Rm = qr_forward(tmp)
            hnew = updateleft(hs[s], Q, Ws[s], Q)
            v = expo_forward("c", -dt / 2, Rm, None, hnew, hs[s + 1])
            r.update(Q=Q, R=Rm, hnew=hnew, v=v)
            tape.append(r)
            mps[s] = Q
            mps[s + 1] = np.tensordot(v, mps[s + 1], axes=([1], [0]))
            hs[s + 1] = hnew
        s = L - 1                               # tdvp.jl:41-43
        tape.append({"kind": "last", "s": s, "x": mps[s], "Le": hs[s], "Re": hs[s + 1]})
        mps[s] = expo_forward("ac", dt, mps[s], Ws[s], hs[s], hs[s + 1])
        for s in range(L - 2, -1, -1):          # _rightsweep! (tdvp.jl:53-68)
            Lm, Qp, pair = lq_forward(mps[s + 1])
            hnew = updateright(hs[s + 2], Qp, Ws[s + 1], Qp)
            v = expo_forward("c", -dt / 2, Lm, None, hs[s + 1], hnew)
            Av = np.tensordot(mps[s], v, axes=([2], [0]))
            tape.append({"kind": "right", "s": s, "pair": pair, "Lm": Lm, "Qp": Qp,
                         "hold": hs[s + 2], "Lc": hs[s + 1], "Le": hs[s], "hnew": hnew, "v": v,
                         "A": mps[s], "Av": Av})
            mps[s + 1] = Qp
            hs[s + 1] = hnew
            mps[s] = expo_forward("ac", dt / 2, Av, Ws[s], hs[s], hnew)
    return mps, {"init": init, "steps": tape, "dt": dt, "L": L}


def observable(mps, site, Op):
    """(n1, n0) = (<psi|O_site|psi>, <psi|psi>) by right-to-left overlap chains
    (operators/expecs.jl:29-55 with a one-site term); ``site`` 0-based."""
    d = mps[0].shape[1]
    I = np.eye(d).reshape(1, d, 1, d).astype(np.complex128)
    O = np.asarray(Op, dtype=np.complex128).reshape(1, d, 1, d)
    n1 = np.ones((1, 1, 1), dtype=np.complex128)
    n0 = np.ones((1, 1, 1), dtype=np.complex128)
    for i in range(len(mps) - 1, -1, -1):
        n1 = updateright(n1, mps[i], O if i == site else I, mps[i])
        n0 = updateright(n0, mps[i], I, mps[i])
    return n1.reshape(-1)[0], n0.reshape(-1)[0]


def observable_backward(mps, site, Op):
    """MPS cotangents of L = Re(n1 / n0)."""
    L = len(mps)
    d = mps[0].shape[1]
    I = np.eye(d).reshape(1, d, 1, d).astype(np.complex128)
    O = np.asarray(Op, dtype=np.complex128).reshape(1, d, 1, d)
    h1 = {L: np.ones((1, 1, 1), dtype=np.complex128)}
    h0 = {L: np.ones((1, 1, 1), dtype=np.complex128)}
    for i in range(L - 1, -1, -1):
        h1[i] = updateright(h1[i + 1], mps[i], O if i == site else I, mps[i])
        h0[i] = updateright(h0[i + 1], mps[i], I, mps[i])
    n1, n0 = h1[0].reshape(-1)[0], h0[0].reshape(-1)[0]
    b1 = np.full((1, 1, 1), np.conj(1.0 / n0), dtype=np.complex128)
    b0 = np.full((1, 1, 1), np.conj(-n1 / n0 ** 2), dtype=np.complex128)
    grads = [None] * L
    for i in range(L):
        hb1, Ab1, _, Bb1 = updateright_backward(b1, h1[i + 1], mps[i], O if i == site else I,
                                                mps[i])
        hb0, Ab0, _, Bb0 = updateright_backward(b0, h0[i + 1], mps[i], I, mps[i])
        grads[i] = Ab1 + Bb1 + Ab0 + Bb0
        b1, b0 = hb1, hb0
    return grads


def tdvp1_backward(Ws, tape, mps_bar):
    """Reverse of tdvp1_forward: given the cotangents of the final MPS, returns
    the cotangent of every site's MPO tensor (Wbar)."""
    L, dt = tape["L"], tape["dt"]
    Wb = [np.zeros(W.shape, dtype=np.complex128) for W in Ws]
    mb = [np.array(g, dtype=np.complex128) for g in mps_bar]
    hb = [None] * (L + 1)

    def add(i, g):
        hb[i] = g if hb[i] is None else hb[i] + g

    def pop(i):
        g = hb[i]
        hb[i] = None
        return g

    for r in reversed(tape["steps"]):
        s = r["s"]
        if r["kind"] == "right":
            # mps[s] = expo_ac(dt/2, Av; W_s, hs[s], hnew)
            xb, lb, wb, rb = expo_backward("ac", dt / 2, r["Av"], mb[s], Ws[s], r["Le"], r["hnew"])
            Wb[s] += wb
            add(s, lb)
            add(s + 1, rb)
            Avb = xb
            # Av = A v
            Dl, d, k = r["A"].shape
            Am = r["A"].reshape(Dl * d, k, order="F")
            Cm = Avb.reshape(Dl * d, -1, order="F")
            mb[s] = (Cm @ r["v"].conj().T).reshape(r["A"].shape, order="F")
            vb = Am.conj().T @ Cm
            # hs[s+1] = hnew
            hnb = pop(s + 1)
            # v = expo_c(-dt/2, Lm; hs[s], hnew)
            xb2, lb2, _, rb2 = expo_backward("c", -dt / 2, r["Lm"], vb, None, r["Lc"], r["hnew"])
            Lmb = xb2
            add(s + 1, lb2)          # the left environment hs[s+1] before it was replaced
            hnb = hnb + rb2 if hnb is not None else rb2
            # hnew = updateright(hs[s+2], Qp, W_{s+1}, Qp)
            hold_b, Ab, wb, Bb = updateright_backward(hnb, r["hold"], r["Qp"], Ws[s + 1], r["Qp"])
            add(s + 2, hold_b)
            Wb[s + 1] += wb
            Qpb = Ab + Bb + mb[s + 1]
            # (Lm, Qp) = lq(mps[s+1])
            mb[s + 1] = lq_backward(r["pair"], Lmb, Qpb).reshape(-1, Ws[s + 1].shape[1],
                                                                  r["Qp"].shape[2], order="F")
        elif r["kind"] == "last":
            xb, lb, wb, rb = expo_backward("ac", dt, r["x"], mb[s], Ws[s], r["Le"], r["Re"])
            mb[s] = xb
            Wb[s] += wb
            add(s, lb)
            add(s + 1, rb)
        else:   # left
            hnb = pop(s + 1)                     # hs[s+1] = hnew
            # mps[s+1] = v B
            Cb = mb[s + 1]
            B = r["B"]
            k = r["v"].shape[0]
            Bm = B.reshape(B.shape[0], -1, order="F")
            Cm = Cb.reshape(k, -1, order="F")
            vb = Cm @ Bm.conj().T
            mb[s + 1] = (r["v"].conj().T @ Cm).reshape(B.shape, order="F")
            Qb = mb[s]                           # mps[s] = Q
            mb[s] = None
            # v = expo_c(-dt/2, R; hnew, hs[s+1])
            Rb, lb, _, rb = expo_backward("c", -dt / 2, r["R"], vb, None, r["hnew"], r["Re"])
            hnb = hnb + lb if hnb is not None else lb
            add(s + 1, rb)
            # hnew = updateleft(hs[s], Q, W_s, Q)
            hold_b, Ab, wb, Bb = updateleft_backward(hnb, r["Le"], r["Q"], Ws[s], r["Q"])
            add(s, hold_b)
            Wb[s] += wb
            Qb = Qb + Ab + Bb
            # (Q, R) = qr(tmp)
            Dl, d, k2 = r["Q"].shape
            tmpb = qr_backward(r["Q"].reshape(Dl * d, k2, order="F"), r["R"],
                               Qb.reshape(Dl * d, k2, order="F"), Rb)
            tmpb = tmpb.reshape(Dl, d, -1, order="F")
            # tmp = expo_ac(dt/2, x; W_s, hs[s], hs[s+1])
            xb, lb, wb, rb = expo_backward("ac", dt / 2, r["x"], tmpb, Ws[s], r["Le"], r["Re"])
            mb[s] = xb
            Wb[s] += wb
            add(s, lb)
            add(s + 1, rb)
    for i, hnext, A in reversed(tape["init"]):
        g = pop(i)
        if g is None:
            continue
        hold_b, _, wb, _ = updateright_backward(g, hnext, A, Ws[i], A)
        add(i + 1, hold_b)
        Wb[i] += wb
    return Wb


def loss_and_grad(h, mps0, dt, nsteps, site, Op):
    """L = Re <Op_site>(T) after nsteps TDVP1 steps of H = -sum Z Z - sum h_i X_i
    from mps0, and dL/dh (real)."""
    Ws = [tfi_site_tensor(hi) for hi in h]
    mps, tape = tdvp1_forward(Ws, mps0, dt, nsteps)
    n1, n0 = observable(mps, site, Op)
    mps_bar = observable_backward(mps, site, Op)
    Wb = tdvp1_backward(Ws, tape, mps_bar)
    G = dW_dh()
    grad = np.array([np.real(np.sum(np.conj(Wb[i]) * G)) for i in range(len(h))])
    return float(np.real(n1 / n0)), grad


def fd_grad(h, mps0, dt, nsteps, site, Op, step=1e-5):
    """Central finite differences of the same forward map."""
    g = np.zeros(len(h))
    for i in range(len(h)):
        hp = np.array(h, dtype=float)
        hm = np.array(h, dtype=float)
        hp[i] += step
        hm[i] -= step
        Wp = [tfi_site_tensor(v) for v in hp]
        Wm = [tfi_site_tensor(v) for v in hm]
        mp, _ = tdvp1_forward(Wp, mps0, dt, nsteps)
        mm, _ = tdvp1_forward(Wm, mps0, dt, nsteps)
        a1, a0 = observable(mp, site, Op)
        b1, b0 = observable(mm, site, Op)
        g[i] = (np.real(a1 / a0) - np.real(b1 / b0)) / (2 * step)
    return g
