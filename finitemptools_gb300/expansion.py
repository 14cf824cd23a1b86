"""Single-site algorithms with subspace expansion and two-site TDVP on the device:
OptimalExpansion (algorithms/expansion/optimalexpand.jl:12-69), DMRG1S
(algorithms/dmrg.jl:148-215, the reference's default ground-state algorithm),
TDVP2 (algorithms/tdvp.jl:71-138) and TDVP1S (tdvp.jl:140-222).

OptimalExpansion enlarges a bond with the leading singular directions of the
two-site residual projected onto the complements of the current site tensors,
NL' * ac2_prime(A B) * NR'.  The reference builds NL = leftnull(A) and
NR = rightnull(B) explicitly.  Here the projectors (I - Q Q^H) and
(I - Q'^H Q') are applied instead, with Q and Q' the QR / LQ factors of A and B.
The projected matrix has the singular values of NL' M NR', and its singular
vectors are NL U1 and V1 NR, which is all the expansion uses, so no null-space
basis is ever formed.
"""

import ctypes

import numpy as np

from ._native import lib
from .auxiliary import (MPSTruncation, default_truncation, gemm, leftorth, rightorth, scale_cols,
                        scale_rows, stable_tsvd)
from .derivatives import HeffOp
from .device import DeviceTensor
from .envs import updateleft_, updateright_
from .excited import projectors1

__all__ = ["OptimalExpansion", "default_expansion", "DMRG1S", "TDVP2", "TDVP1S",
           "right_expansion_", "left_expansion_", "dmrg1s_leftsweep_", "dmrg1s_rightsweep_",
           "tdvp2_sweep_", "tdvp1s_sweep_"]


class OptimalExpansion:
    """struct OptimalExpansion (optimalexpand.jl:4).

    ``cap`` (not in the reference, off by default): add at most trunc.D - D new
    directions.  The expanded matrix [B ; V1 NR] has orthonormal rows, so all
    its singular values are 1; once D + k exceeds trunc.D, the reference's
    truncation of it keeps an arbitrary D-dimensional subspace and drops part of
    the state, and DMRG1S stalls near 1e-3 (XXZ L=20, D=64).  With the cap a
    saturated bond is not expanded, and the sweep converges like DMRG2."""

    def __init__(self, cap=False):
        self.cap = bool(cap)


def default_expansion():
    return OptimalExpansion()


class DMRG1S:
    """@with_kw struct DMRG1S (dmrg.jl:148-156) plus the device options."""

    def __init__(self, maxiter=100, tol=1e-12, eig_maxiter=10, eig_tol=1e-12, verbosity=1,
                 trunc=None, expan=None, precision="fp64", reorth=False):
        self.maxiter, self.tol = maxiter, tol
        self.eig_maxiter, self.eig_tol = eig_maxiter, eig_tol
        self.verbosity = verbosity
        self.trunc = trunc if trunc is not None else default_truncation()
        self.expan = expan if expan is not None else default_expansion()
        self.precision, self.reorth = precision, reorth


class TDVP2:
    """struct TDVP2 (tdvp.jl:71-79); stepsize -1j*dt for real time."""

    def __init__(self, stepsize, exptol=1e-8, ishermitian=False, verbosity=1, trunc=None,
                 krylovdim=30, precision="fp64"):
        self.stepsize, self.exptol, self.ishermitian = stepsize, exptol, ishermitian
        self.verbosity = verbosity
        self.trunc = trunc if trunc is not None else default_truncation()
        self.krylovdim, self.precision = krylovdim, precision


class TDVP1S:
    """struct TDVP1S (tdvp.jl:140-155)."""

    def __init__(self, stepsize, exptol=1e-8, ishermitian=False, verbosity=1, trunc=None,
                 expan=None, krylovdim=30, precision="fp64"):
        self.stepsize, self.exptol, self.ishermitian = stepsize, exptol, ishermitian
        self.verbosity = verbosity
        self.trunc = trunc if trunc is not None else default_truncation()
        self.expan = expan if expan is not None else default_expansion()
        self.krylovdim, self.precision = krylovdim, precision


# ------------------------------------------------------------------ helpers
def _copy2d(src, m, n, lds, dst, ldd, dst_row=0, dst_col=0):
    """dst[dst_row:dst_row+m, dst_col:dst_col+n] = src (column-major blocks)."""
    h = src.h
    cp = src.code == 1
    ps = src.size if cp else 0
    pd = dst.size if cp else 0
    off = (dst_row + ldd * dst_col) * 8
    h.check(lib().fmpt_copy2d(h.ptr, src.code, int(m), int(n), src.ptr, int(lds), ps,
                              dst.ptr + off, int(ldd), pd))


def _complement(M, m, n, QL, QR):
    """(I - QL QL^H) M (I - QR^H QR) for an m x n device matrix M (in place)."""
    rl = QL.shape[1]
    t = gemm(QL, M, (rl, n), rl, n, m, ta="C", lda=m, ldb=m)
    gemm(QL, t, None, m, n, rl, alpha=-1.0, beta=1.0, C=M, lda=m, ldb=rl, ldc=m)
    rr = QR.shape[0]
    t = gemm(M, QR, (m, rr), m, rr, n, tb="C", lda=m, ldb=rr)
    gemm(t, QR, None, m, n, rr, alpha=-1.0, beta=1.0, C=M, lda=m, ldb=rr, ldc=m)
    return M


def _residual_directions(m, site, trunc, cap=False):
    """Truncated SVD of NL' * ac2_prime(mps[site] mps[site+1]) * NR' in the full
    space: (u = NL U1 [Dl*d x k], v = V1 NR [k x d*Dr]) or None."""
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    A, B = mps[site], mps[site + 1]
    Dl, d1, D = A.shape
    _, d2, Dr = B.shape
    # dimensions of leftnull(A) and rightnull(B) (full-rank site tensors): nothing to
    # expand into when either is empty; at most min of the two directions otherwise
    cl, cr = Dl * d1 - D, d2 * Dr - D
    room = trunc.D - D if cap else trunc.D
    if cl <= 0 or cr <= 0 or room <= 0:
        return None
    trunc = MPSTruncation(min(trunc.D, cl, cr, room), trunc.eps, trunc.verbosity)
    x2 = gemm(A, B, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, D)
    op = HeffOp("ac2", hs[site], hs[site + 2], W1=mpo[site], W2=mpo[site + 1], dtype=A.dtype)
    ac2 = op(x2)
    del op
    QL, _ = leftorth(A, Dl * d1, D)
    _, QR = rightorth(B, D, d2 * Dr)
    QR.view_as((QR.shape[0], d2 * Dr))
    M = ac2.view_as((Dl * d1, d2 * Dr))
    _complement(M, Dl * d1, d2 * Dr, QL, QR)
    u, s, vt, _ = stable_tsvd(M, Dl * d1, d2 * Dr, trunc)
    return u, s, vt


def right_expansion_(m, site, expan, trunc):
    """right_expansion! (optimalexpand.jl:42-69): enlarge the bond between
    site and site+1 from the right, during a left-to-right sweep."""
    mps = m.mps
    A, B = mps[site], mps[site + 1]
    Dl, d1, D = A.shape
    _, d2, Dr = B.shape
    r = _residual_directions(m, site, trunc, getattr(expan, "cap", False))
    k = 0 if r is None else r[2].shape[0]
    # b = [B ; V1 NR]  ((D + k) x (d2 Dr))
    bcat = DeviceTensor((D + k, d2 * Dr), B.dtype, B.h)
    _copy2d(B, D, d2 * Dr, D, bcat, D + k)
    if k:
        _copy2d(r[2], k, d2 * Dr, k, bcat, D + k, dst_row=D)
    u2, s2, v2, _ = stable_tsvd(bcat, D + k, d2 * Dr, trunc)
    kk = s2.shape[0]
    mps[site + 1] = v2.view_as((kk, d2, Dr))
    # a * u * s with a = [A | 0]: only the first D rows of u meet nonzero columns
    new = gemm(A, u2, (Dl, d1, kk), Dl * d1, kk, D, lda=Dl * d1, ldb=D + k)
    mps[site] = scale_cols(new, Dl * d1, kk, s2)
    updateright_(m, site + 1)


def left_expansion_(m, site, expan, trunc):
    """left_expansion! (optimalexpand.jl:12-38): enlarge the bond between
    site-1 and site from the left, during a right-to-left sweep."""
    mps = m.mps
    A, B = mps[site - 1], mps[site]
    Dl, d1, D = A.shape
    _, d2, Dr = B.shape
    r = _residual_directions(m, site - 1, trunc, getattr(expan, "cap", False))
    k = 0 if r is None else r[0].shape[1]
    # a = [A | NL U1]  ((Dl d1) x (D + k)), columns are contiguous
    acat = DeviceTensor((Dl * d1, D + k), A.dtype, A.h)
    _copy2d(A, Dl * d1, D, Dl * d1, acat, Dl * d1)
    if k:
        _copy2d(r[0], Dl * d1, k, Dl * d1, acat, Dl * d1, dst_col=D)
    u2, s2, v2, _ = stable_tsvd(acat, Dl * d1, D + k, trunc)
    kk = s2.shape[0]
    mps[site - 1] = u2.view_as((Dl, d1, kk))
    # s * v * b with b = [B ; 0]: only the first D columns of v meet nonzero rows.
    # Those columns are copied out first: a complex operand's imaginary plane sits
    # at ld x (columns used) in fmpt_gemm, and v's plane holds D + k columns.
    if k:
        vD = DeviceTensor((kk, D), v2.dtype, v2.h)
        _copy2d(v2, kk, D, kk, vD, kk)
        v2 = vD
    new = gemm(v2, B, (kk, d2, Dr), kk, d2 * Dr, D, lda=kk, ldb=D)
    mps[site] = scale_rows(new, kk, d2 * Dr, s2)
    updateleft_(m, site - 1)


# -------------------------------------------------------------------- DMRG1S
def dmrg1s_leftsweep_(m, alg):
    """leftsweep!(m, ::DMRG1S) (dmrg.jl:158-186); projected caches as in
    dmrgexcited.jl:153-184."""
    from .algorithms import _galerkin, _start_vector
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    Es, delta = [], 0.0
    for site in range(1, len(mps)):
        right_expansion_(m, site, alg.expan, alg.trunc)
        A = mps[site]
        op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                    dtype=A.dtype)
        x0 = _start_vector(op, A, projectors1(m, site))
        E, vec, _, _ = op.lanczos(x0, alg.eig_maxiter, alg.eig_tol, alg.reorth)
        del op
        Es.append(E)
        delta = max(delta, _galerkin(m, site, alg.precision))
        Dl, d, Dr = A.shape
        Q, R = leftorth(vec, Dl * d, Dr)
        r = Q.shape[1]
        mps[site] = Q.view_as((Dl, d, r))
        B = mps[site + 1]
        mps[site + 1] = gemm(R, B, (r, B.shape[1], B.shape[2]), r, B.shape[1] * B.shape[2], Dr)
        updateleft_(m, site)
    return Es, delta


def dmrg1s_rightsweep_(m, alg):
    """rightsweep!(m, ::DMRG1S) (dmrg.jl:188-215); projected caches as in
    dmrgexcited.jl:186-216."""
    from .algorithms import _galerkin, _start_vector
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    Es, delta = [], 0.0
    for site in range(len(mps), 1, -1):
        left_expansion_(m, site, alg.expan, alg.trunc)
        A = mps[site]
        op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                    dtype=A.dtype)
        x0 = _start_vector(op, A, projectors1(m, site))
        E, vec, _, _ = op.lanczos(x0, alg.eig_maxiter, alg.eig_tol, alg.reorth)
        del op
        Es.append(E)
        delta = max(delta, _galerkin(m, site, alg.precision))
        Dl, d, Dr = A.shape
        Lm, Q = rightorth(vec, Dl, d * Dr)
        r = Q.shape[0]
        mps[site] = Q.view_as((r, d, Dr))
        P = mps[site - 1]
        mps[site - 1] = gemm(P, Lm, (P.shape[0], P.shape[1], r), P.shape[0] * P.shape[1], r, Dl)
        updateright_(m, site)
    return Es, delta


# --------------------------------------------------------------------- TDVP2
def _expo(kind, m, site, t, x, alg, W2=None):
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    if kind == "ac2":
        op = HeffOp("ac2", hs[site], hs[site + 2], W1=mpo[site], W2=mpo[site + 1],
                    precision=alg.precision, dtype=x.dtype)
    else:
        op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                    dtype=x.dtype)
    y = op.exponentiate(t, x, alg.exptol / abs(t), alg.krylovdim)
    del op
    return y


def tdvp2_sweep_(m, alg):
    """sweep!(m, ::TDVP2) = _leftsweep! + _rightsweep! (tdvp.jl:82-138)."""
    from .transfer import updateleft, updateright
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    dt = alg.stepsize
    L = len(mps)
    envp = "fp64" if mps[1].dtype == np.complex128 else alg.precision
    for site in range(1, L - 1):
        A, B = mps[site], mps[site + 1]
        Dl, d1, D = A.shape
        _, d2, Dr = B.shape
        x2 = gemm(A, B, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, D)
        x2 = _expo("ac2", m, site, dt / 2, x2, alg)
        u, s, vt, _ = stable_tsvd(x2, Dl * d1, d2 * Dr, alg.trunc)
        k = s.shape[0]
        mps[site] = u.view_as((Dl, d1, k))
        sv = scale_rows(vt, k, d2 * Dr, s).view_as((k, d2, Dr))
        hs[site + 1] = updateleft(hs[site], mps[site], mpo[site], mps[site], envp)
        mps[site + 1] = _expo("ac", m, site + 1, -dt / 2, sv, alg)
    site = L - 1
    A, B = mps[site], mps[site + 1]
    Dl, d1, D = A.shape
    _, d2, Dr = B.shape
    x2 = gemm(A, B, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, D)
    x2 = _expo("ac2", m, site, dt, x2, alg)
    u, s, vt, _ = stable_tsvd(x2, Dl * d1, d2 * Dr, alg.trunc)
    k = s.shape[0]
    mps[site] = scale_cols(u, Dl * d1, k, s).view_as((Dl, d1, k))
    mps[site + 1] = vt.view_as((k, d2, Dr))
    hs[site + 1] = updateright(hs[site + 2], mps[site + 1], mpo[site + 1], mps[site + 1], envp)
    mps.s[site + 1] = s
    for site in range(L - 2, 0, -1):
        mps[site + 1] = _expo("ac", m, site + 1, -dt / 2, mps[site + 1], alg)
        A, B = mps[site], mps[site + 1]
        Dl, d1, D = A.shape
        _, d2, Dr = B.shape
        x2 = gemm(A, B, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, D)
        x2 = _expo("ac2", m, site, dt / 2, x2, alg)
        u, s, vt, _ = stable_tsvd(x2, Dl * d1, d2 * Dr, alg.trunc)
        k = s.shape[0]
        mps[site] = scale_cols(u, Dl * d1, k, s).view_as((Dl, d1, k))
        mps[site + 1] = vt.view_as((k, d2, Dr))
        hs[site + 1] = updateright(hs[site + 2], mps[site + 1], mpo[site + 1], mps[site + 1],
                                   envp)
        mps.s[site + 1] = s


# -------------------------------------------------------------------- TDVP1S
def tdvp1s_sweep_(m, alg):
    """sweep!(m, ::TDVP1S) (tdvp.jl:158-217): TDVP1 with a right expansion before
    every left-sweep site and a left expansion in the right sweep."""
    from .transfer import updateleft, updateright
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    dt = alg.stepsize
    L = len(mps)
    envp = "fp64" if mps[1].dtype == np.complex128 else alg.precision
    for site in range(1, L):
        right_expansion_(m, site, alg.expan, alg.trunc)
        A = mps[site]
        tmp = _expo("ac", m, site, dt / 2, A, alg)
        Dl, d, Dr = A.shape
        Q, v = leftorth(tmp, Dl * d, Dr)
        r = Q.shape[1]
        mps[site] = Q.view_as((Dl, d, r))
        hnew = updateleft(hs[site], mps[site], mpo[site], mps[site], envp)
        opc = HeffOp("c", hnew, hs[site + 1], precision=alg.precision, dtype=A.dtype)
        v = opc.exponentiate(-dt / 2, v, alg.exptol / abs(dt / 2), alg.krylovdim)
        del opc
        B = mps[site + 1]
        mps[site + 1] = gemm(v, B, (r, B.shape[1], B.shape[2]), r, B.shape[1] * B.shape[2], Dr)
        hs[site + 1] = hnew
    site = L
    mps[site] = _expo("ac", m, site, dt, mps[site], alg)
    for site in range(L - 1, 0, -1):
        B = mps[site + 1]
        Dl, d, Dr = B.shape
        v, Q = rightorth(B, Dl, d * Dr)
        r = Q.shape[0]
        mps[site + 1] = Q.view_as((r, d, Dr))
        hnew = updateright(hs[site + 2], mps[site + 1], mpo[site + 1], mps[site + 1], envp)
        opc = HeffOp("c", hs[site + 1], hnew, precision=alg.precision, dtype=B.dtype)
        v = opc.exponentiate(-dt / 2, v, alg.exptol / abs(dt / 2), alg.krylovdim)
        del opc
        hs[site + 1] = hnew
        P = mps[site]
        mps[site] = gemm(P, v, (P.shape[0], P.shape[1], r), P.shape[0] * P.shape[1], r, Dl)
        if site > 1:
            left_expansion_(m, site, alg.expan, alg.trunc)
        mps[site] = _expo("ac", m, site, dt / 2, mps[site], alg)
