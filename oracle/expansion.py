"""Restatement of the single-site algorithms with subspace expansion and of
two-site TDVP (test infrastructure only: the product never imports this module).

- OptimalExpansion: algorithms/expansion/optimalexpand.jl:12-69, with explicit
  null spaces (leftnull / rightnull as orthonormal complements);
- DMRG1S: algorithms/dmrg.jl:148-215;
- TDVP2:  algorithms/tdvp.jl:82-138;
- TDVP1S: algorithms/tdvp.jl:158-217.
Site numbers are 1-based as in the reference; OracleEnv stores 0-based lists.
"""

import numpy as np
import scipy.linalg

from .algorithms import _galerkin
from .core import ac2_prime, ac_prime, c_prime, krylov_exponentiate, leftorth_qr, rightorth_lq
from .core import stable_tsvd, updateleft, updateright

__all__ = ["right_expansion", "left_expansion", "dmrg1s_sweep", "tdvp2_sweep", "tdvp1s_sweep"]


def _leftnull(A):
    """Orthonormal basis (rows of A's codomain) of the complement of range(A)."""
    Dl, d, D = A.shape
    M = A.reshape(Dl * d, D, order="F")
    return scipy.linalg.null_space(M.conj().T)            # (Dl d) x r


def _rightnull(B):
    """Orthonormal rows spanning the complement of B's row space."""
    D, d, Dr = B.shape
    M = B.reshape(D, d * Dr, order="F")
    return scipy.linalg.null_space(M).conj().T            # r x (d Dr)


def _residual(env, site, trunc, cap=False):
    A, B = env.mps[site - 1], env.mps[site]
    if cap:
        # not in the reference: at most trunc.D - D new directions
        room = trunc.D - A.shape[2]
        if room <= 0:
            return None
        trunc = type(trunc)(min(trunc.D, room), trunc.eps)
    x2 = np.tensordot(A, B, axes=([2], [0]))
    ac2 = ac2_prime(x2, env.mpo[site - 1], env.mpo[site], env.hstorage[site - 1],
                    env.hstorage[site + 1])
    Dl, d1, d2, Dr = ac2.shape
    NL, NR = _leftnull(A), _rightnull(B)
    if NL.shape[1] == 0 or NR.shape[0] == 0:
        return None
    inter = NL.conj().T @ ac2.reshape(Dl * d1, d2 * Dr, order="F") @ NR.conj().T
    U1, S1, V1, _ = stable_tsvd(inter, trunc)
    return NL @ U1, V1 @ NR


def right_expansion(env, site, trunc, cap=False):
    """right_expansion! (optimalexpand.jl:42-69)."""
    A, B = env.mps[site - 1], env.mps[site]
    Dl, d1, D = A.shape
    _, d2, Dr = B.shape
    r = _residual(env, site, trunc, cap)
    Bm = B.reshape(D, d2 * Dr, order="F")
    bcat = Bm if r is None else np.vstack([Bm, r[1]])
    u, s, v, _ = stable_tsvd(bcat, trunc)
    k = s.shape[0]
    env.mps[site] = v.reshape(k, d2, Dr, order="F")
    Am = A.reshape(Dl * d1, D, order="F")
    env.mps[site - 1] = ((Am @ u[:D, :]) * s[None, :]).reshape(Dl, d1, k, order="F")
    env.updateright_(site + 1)


def left_expansion(env, site, trunc, cap=False):
    """left_expansion! (optimalexpand.jl:12-38)."""
    A, B = env.mps[site - 2], env.mps[site - 1]
    Dl, d1, D = A.shape
    _, d2, Dr = B.shape
    r = _residual(env, site - 1, trunc, cap)
    Am = A.reshape(Dl * d1, D, order="F")
    acat = Am if r is None else np.hstack([Am, r[0]])
    u, s, v, _ = stable_tsvd(acat, trunc)
    k = s.shape[0]
    env.mps[site - 2] = u.reshape(Dl, d1, k, order="F")
    Bm = B.reshape(D, d2 * Dr, order="F")
    env.mps[site - 1] = ((s[:, None] * v[:, :D]) @ Bm).reshape(k, d2, Dr, order="F")
    env.updateleft_(site - 1)


def _lanczos(env, site, eig_maxiter, eig_tol):
    from .core import simple_lanczos_solver
    A = env.mps[site - 1]
    W, Le, Re = env.mpo[site - 1], env.hstorage[site - 1], env.hstorage[site]

    def f(v):
        return ac_prime(v.reshape(A.shape, order="F"), W, Le, Re).ravel(order="F")

    E, vec, _, _ = simple_lanczos_solver(f, A.ravel(order="F"), eig_maxiter, eig_tol)
    return E, vec.reshape(A.shape, order="F")


def dmrg1s_sweep(env, trunc, eig_maxiter=10, eig_tol=1e-12, cap=False):
    """sweep!(m, ::DMRG1S): leftsweep! + rightsweep! (dmrg.jl:158-215)."""
    L = len(env.mps)
    Es, delta = [], 0.0
    for site in range(1, L):
        right_expansion(env, site, trunc, cap)
        E, vec = _lanczos(env, site, eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, _galerkin(env, site, env.mps[site - 1]))
        Q, R = leftorth_qr(vec)
        env.mps[site - 1] = Q
        env.mps[site] = np.tensordot(R, env.mps[site], axes=([1], [0]))
        env.updateleft_(site)
    for site in range(L, 1, -1):
        left_expansion(env, site, trunc, cap)
        E, vec = _lanczos(env, site, eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, _galerkin(env, site, env.mps[site - 1]))
        Lm, Q = rightorth_lq(vec)
        env.mps[site - 1] = Q
        env.mps[site - 2] = np.tensordot(env.mps[site - 2], Lm, axes=([2], [0]))
        env.updateright_(site)
    return Es, delta


def _expo(f, t, x, exptol, krylovdim):
    shape = x.shape
    y = krylov_exponentiate(lambda v: f(v.reshape(shape, order="F")).ravel(order="F"), t,
                            x.ravel(order="F"), tol=exptol / abs(t), krylovdim=krylovdim)
    return y.reshape(shape, order="F")


def tdvp2_sweep(env, dt, trunc, exptol=1e-8, krylovdim=30):
    """sweep!(m, ::TDVP2) (tdvp.jl:82-138)."""
    mps, mpo, hs = env.mps, env.mpo, env.hstorage
    L = len(mps)

    def ac2(site):
        return lambda x: ac2_prime(x, mpo[site - 1], mpo[site], hs[site - 1], hs[site + 1])

    def ac1(site):
        return lambda x: ac_prime(x, mpo[site - 1], hs[site - 1], hs[site])

    for site in range(1, L - 1):
        x2 = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
        x2 = _expo(ac2(site), dt / 2, x2, exptol, krylovdim)
        Dl, d1, d2, Dr = x2.shape
        u, s, v, _ = stable_tsvd(x2.reshape(Dl * d1, d2 * Dr, order="F"), trunc)
        k = s.shape[0]
        mps[site - 1] = u.reshape(Dl, d1, k, order="F")
        sv = (s[:, None] * v).reshape(k, d2, Dr, order="F")
        hs[site] = updateleft(hs[site - 1], mps[site - 1], mpo[site - 1], mps[site - 1])
        mps[site] = _expo(ac1(site + 1), -dt / 2, sv, exptol, krylovdim)
    site = L - 1
    x2 = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
    x2 = _expo(ac2(site), dt, x2, exptol, krylovdim)
    Dl, d1, d2, Dr = x2.shape
    u, s, v, _ = stable_tsvd(x2.reshape(Dl * d1, d2 * Dr, order="F"), trunc)
    k = s.shape[0]
    mps[site - 1] = (u * s[None, :]).reshape(Dl, d1, k, order="F")
    mps[site] = v.reshape(k, d2, Dr, order="F")
    hs[site] = updateright(hs[site + 1], mps[site], mpo[site], mps[site])
    for site in range(L - 2, 0, -1):
        mps[site] = _expo(ac1(site + 1), -dt / 2, mps[site], exptol, krylovdim)
        x2 = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
        x2 = _expo(ac2(site), dt / 2, x2, exptol, krylovdim)
        Dl, d1, d2, Dr = x2.shape
        u, s, v, _ = stable_tsvd(x2.reshape(Dl * d1, d2 * Dr, order="F"), trunc)
        k = s.shape[0]
        mps[site - 1] = (u * s[None, :]).reshape(Dl, d1, k, order="F")
        mps[site] = v.reshape(k, d2, Dr, order="F")
        hs[site] = updateright(hs[site + 1], mps[site], mpo[site], mps[site])


def tdvp1s_sweep(env, dt, trunc, exptol=1e-8, krylovdim=30):
    """sweep!(m, ::TDVP1S) (tdvp.jl:158-217)."""
    mps, mpo, hs = env.mps, env.mpo, env.hstorage
    L = len(mps)
    for site in range(1, L):
        right_expansion(env, site, trunc)
        W, Le, Re = mpo[site - 1], hs[site - 1], hs[site]
        tmp = _expo(lambda x: ac_prime(x, W, Le, Re), dt / 2, mps[site - 1], exptol, krylovdim)
        Q, v = leftorth_qr(tmp)
        mps[site - 1] = Q
        hnew = updateleft(hs[site - 1], Q, W, Q)
        v = _expo(lambda x: c_prime(x, hnew, Re), -dt / 2, v, exptol, krylovdim)
        mps[site] = np.tensordot(v, mps[site], axes=([1], [0]))
        hs[site] = hnew
    site = L
    mps[site - 1] = _expo(lambda x: ac_prime(x, mpo[site - 1], hs[site - 1], hs[site]), dt,
                          mps[site - 1], exptol, krylovdim)
    for site in range(L - 1, 0, -1):
        v, Q = rightorth_lq(mps[site])
        mps[site] = Q
        hnew = updateright(hs[site + 1], Q, mpo[site], Q)
        Le = hs[site]
        v = _expo(lambda x: c_prime(x, Le, hnew), -dt / 2, v, exptol, krylovdim)
        hs[site] = hnew
        mps[site - 1] = np.tensordot(mps[site - 1], v, axes=([2], [0]))
        if site > 1:
            left_expansion(env, site, trunc)
        W2, Le2, Re2 = mpo[site - 1], hs[site - 1], hs[site]
        mps[site - 1] = _expo(lambda x: ac_prime(x, W2, Le2, Re2), dt / 2, mps[site - 1], exptol,
                              krylovdim)
