"""Restatement of the excited-state (projected) DMRG (test infrastructure only:
the product never imports this module).

- ProjectedExpectationCache and its overlap environments:
  envs/finiteenv.jl:96-168;
- overlap transfers of two MPS: mps/transfer.jl:5-20;
- c_proj: algorithms/derivatives.jl:65-67; _c2_prime_2: dmrgexcited.jl:84-86;
- _project!: dmrgexcited.jl:1-6;
- projected DMRG1 / DMRG2 / DMRG1S sweeps: dmrgexcited.jl:9-216.
Site numbers are 1-based as in the reference; the storages are 0-based lists
(cstorages[l][i-1] is the reference's cstorages[l][i]).
"""

import numpy as np

from .algorithms import OracleEnv, _galerkin, bond_dimension, canonicalize, increase_bond
from .core import ac2_prime, ac_prime, leftorth_qr, rightorth_lq, simple_lanczos_solver
from .core import stable_tsvd
from . import expansion as X

__all__ = ["overlap_updateleft", "overlap_updateright", "c_proj", "c2_proj", "project",
           "ProjectedEnv", "pdmrg2_sweep", "pdmrg1_sweep", "pdmrg1s_sweep"]


def overlap_updateleft(hold, A, B):
    """mps/transfer.jl:17-20: hnew[c,d] = sum conj(A[a,s,c]) hold[a,b] B[b,s,d]."""
    t = np.tensordot(hold, B, axes=([1], [0]))                     # [a, s, d]
    return np.tensordot(np.conj(A), t, axes=([0, 1], [0, 1]))      # [c, d]


def overlap_updateright(hold, A, B):
    """mps/transfer.jl:7-10: hnew[c,d] = sum conj(A[c,s,b]) hold[b,e] B[d,s,e]."""
    t = np.tensordot(B, hold, axes=([2], [1]))                     # [d, s, b]
    return np.tensordot(np.conj(A), t, axes=([1, 2], [1, 2]))      # [c, d]


def c_proj(x, cleft, cright):
    """derivatives.jl:65-67: p[a,s,c] = cleft[a,b] x[b,s,e] cright[c,e]."""
    t = np.tensordot(cleft, x, axes=([1], [0]))
    return np.tensordot(t, cright, axes=([2], [1]))


def c2_proj(x1, x2, cleft, cright):
    """_c2_prime_2 (dmrgexcited.jl:84-86):
    p[a,s1,s2,c] = cleft[a,b] x1[b,s1,e] x2[e,s2,f] cright[c,f]."""
    t = np.tensordot(x1, x2, axes=([2], [0]))
    t = np.tensordot(cleft, t, axes=([1], [0]))
    return np.tensordot(t, cright, axes=([3], [1]))


def project(y, ps):
    """_project! (dmrgexcited.jl:1-6): y = y - dot(y, p) p for each p in order,
    with Julia's dot(y, p) = sum conj(y) p."""
    for p in ps:
        y = y - np.vdot(y, p) * p
    return y


class ProjectedEnv(OracleEnv):
    """ProjectedExpectationCache (finiteenv.jl:96-168)."""

    def __init__(self, mpo, mps, projectors, schur=False):
        self.projectors = [[A.copy() for A in p] for p in projectors]
        super().__init__(mpo, mps, schur)
        self.cstorages = [self._init_cstorage(p) for p in self.projectors]

    def _init_cstorage(self, proj):
        """init_cstorage_right! (finiteenv.jl:103-117)."""
        L = len(self.mps)
        if len(proj) != L or self.mps[-1].shape[2] != proj[-1].shape[2]:
            raise ValueError("DimensionMismatch")
        T = np.result_type(self.mps[0], proj[0])
        cs = [None] * (L + 1)
        cs[0] = np.eye(self.mps[0].shape[0], dtype=T)                          # l_LL(psiA)
        cs[L] = np.eye(self.mps[-1].shape[2], proj[-1].shape[2], dtype=T)      # r_RR(psiA, psiB)
        for i in range(L, 1, -1):                                             # Julia L:-1:2
            cs[i - 1] = overlap_updateright(cs[i], self.mps[i - 1], proj[i - 1])
        return cs

    def updateleft_(self, site):
        """updateleft!(::ProjectedExpectationCache, site) (finiteenv.jl:144-149)."""
        super().updateleft_(site)
        for P, cs in zip(self.projectors, self.cstorages):
            cs[site] = overlap_updateleft(cs[site - 1], self.mps[site - 1], P[site - 1])

    def updateright_(self, site):
        """updateright!(::ProjectedExpectationCache, site) (finiteenv.jl:152-157)."""
        super().updateright_(site)
        for P, cs in zip(self.projectors, self.cstorages):
            cs[site - 1] = overlap_updateright(cs[site], self.mps[site - 1], P[site - 1])

    def increase_bond_(self, D):
        """increase_bond!(m::ProjectedExpectationCache; D) (finiteenv.jl:159-168)."""
        if bond_dimension(self.mps) < D:
            self.mps = increase_bond(self.mps, D)
            self.mps, _ = canonicalize(self.mps, normalize=False)
            self.init_hstorage(center=1)
            self.cstorages = [self._init_cstorage(p) for p in self.projectors]

    def p1(self, site):
        """[c_proj(projectors[l][site], cstorages[l][site], cstorages[l][site+1])]."""
        return [c_proj(P[site - 1], cs[site - 1], cs[site])
                for P, cs in zip(self.projectors, self.cstorages)]

    def p2(self, site):
        """[_c2_prime_2(projectors[l][site], projectors[l][site+1], cstorages[l][site],
        cstorages[l][site+2])] (dmrgexcited.jl:97, :125)."""
        return [c2_proj(P[site - 1], P[site], cs[site - 1], cs[site + 1])
                for P, cs in zip(self.projectors, self.cstorages)]


def _pdmrg2_bond(env, site, trunc, eig_maxiter, eig_tol, direction):
    """Bond body of leftsweep!/rightsweep!(::ProjectedExpectationCache, ::DMRG2)
    (dmrgexcited.jl:96-115, :124-145)."""
    mps, mpo, hs = env.mps, env.mpo, env.hstorage
    ps = env.p2(site)
    x2 = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
    shape = x2.shape
    x2 = project(x2, ps)                  # _project!(twositemps, p2) mutates twositemps
    W1, W2, L, R = mpo[site - 1], mpo[site], hs[site - 1], hs[site + 1]

    def f(v):
        y = ac2_prime(v.reshape(shape, order="F"), W1, W2, L, R)
        return project(y, ps).ravel(order="F")

    E, vec, _, _ = simple_lanczos_solver(f, x2.ravel(order="F"), eig_maxiter, eig_tol)
    vec = vec.reshape(shape, order="F")
    Dl, d1, d2, Dr = shape
    u, s, vh, _ = stable_tsvd(vec.reshape(Dl * d1, d2 * Dr, order="F"), trunc)
    s = s / np.linalg.norm(s)
    U = u.reshape(Dl, d1, u.shape[1], order="F")
    V = vh.reshape(vh.shape[0], d2, Dr, order="F")
    usv = np.tensordot(U * s[None, None, :], V, axes=([2], [0]))
    delta = abs(1 - abs(np.vdot(usv, x2)))
    if direction == "left":
        mps[site - 1] = U
        mps[site] = s[:, None, None] * V
        env.updateleft_(site)
    else:
        mps[site - 1] = U * s[None, None, :]
        mps[site] = V
        env.updateright_(site + 1)
    return E, delta


def pdmrg2_sweep(env, trunc, eig_maxiter=10, eig_tol=1e-12):
    """sweep!(::ProjectedExpectationCache, ::DMRG2) (dmrgexcited.jl:89-150, :219-223)."""
    Es, delta = [], 0.0
    L = len(env.mps)
    for site in range(1, L - 1):
        E, dl = _pdmrg2_bond(env, site, trunc, eig_maxiter, eig_tol, "left")
        Es.append(E)
        delta = max(delta, dl)
    for site in range(L - 1, 0, -1):
        E, dl = _pdmrg2_bond(env, site, trunc, eig_maxiter, eig_tol, "right")
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta


def _p_lanczos(env, site, eig_maxiter, eig_tol):
    """Projected one-site eigensolve (dmrgexcited.jl:20-23)."""
    A = env.mps[site - 1]
    W, Le, Re = env.mpo[site - 1], env.hstorage[site - 1], env.hstorage[site]
    ps = env.p1(site)
    x0 = project(A.copy(), ps)

    def f(v):
        return project(ac_prime(v.reshape(A.shape, order="F"), W, Le, Re), ps).ravel(order="F")

    E, vec, _, _ = simple_lanczos_solver(f, x0.ravel(order="F"), eig_maxiter, eig_tol)
    return E, vec.reshape(A.shape, order="F")


def _p1_left(env, site, eig_maxiter, eig_tol):
    E, vec = _p_lanczos(env, site, eig_maxiter, eig_tol)
    g = _galerkin(env, site, env.mps[site - 1])
    Q, R = leftorth_qr(vec)
    env.mps[site - 1] = Q
    env.mps[site] = np.tensordot(R, env.mps[site], axes=([1], [0]))
    env.updateleft_(site)
    return E, g


def _p1_right(env, site, eig_maxiter, eig_tol):
    E, vec = _p_lanczos(env, site, eig_maxiter, eig_tol)
    g = _galerkin(env, site, env.mps[site - 1])
    Lm, Q = rightorth_lq(vec)
    env.mps[site - 1] = Q
    env.mps[site - 2] = np.tensordot(env.mps[site - 2], Lm, axes=([2], [0]))
    env.updateright_(site)
    return E, g


def pdmrg1_sweep(env, D=50, eig_maxiter=10, eig_tol=1e-12):
    """sweep!(::ProjectedExpectationCache, ::DMRG1) (dmrgexcited.jl:9-75)."""
    env.increase_bond_(D)
    Es, delta = [], 0.0
    L = len(env.mps)
    for site in range(1, L):
        E, g = _p1_left(env, site, eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, g)
    for site in range(L, 1, -1):
        E, g = _p1_right(env, site, eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, g)
    return Es, delta


def pdmrg1s_sweep(env, trunc, eig_maxiter=10, eig_tol=1e-12):
    """sweep!(::ProjectedExpectationCache, ::DMRG1S) (dmrgexcited.jl:153-216): the
    expansions update the overlap storages through env.updateleft_/updateright_."""
    Es, delta = [], 0.0
    L = len(env.mps)
    for site in range(1, L):
        X.right_expansion(env, site, trunc)
        E, g = _p1_left(env, site, eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, g)
    for site in range(L, 1, -1):
        X.left_expansion(env, site, trunc)
        E, g = _p1_right(env, site, eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, g)
    return Es, delta
