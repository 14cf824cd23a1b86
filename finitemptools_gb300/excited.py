"""Excited states by projected DMRG on the device: ProjectedExpectationCache
(envs/finiteenv.jl:96-168), the overlap transfers of two MPS
(mps/transfer.jl:5-20), c_proj (algorithms/derivatives.jl:65-67),
_c2_prime_2 and _project! (algorithms/dmrgexcited.jl:1-6, :84-86).

The projected DMRG2 / DMRG1 / DMRG1S sweeps (dmrgexcited.jl:9-216) are the
plain sweeps with two changes, both supplied here: the starting vector is
projected, and the effective Hamiltonian is composed with _project! inside
the library (fmpt_op_set_projectors), so every Lanczos step projects on the
device with its scalars kept there.  The overlap storages
``cstorages[l][i]`` (1-based, length L+1) are [bond of mps, bond of
projector l] matrices.
"""

import numpy as np

from .auxiliary import axpy, dot, gemm
from .device import DeviceTensor
from .envs import ExpectationCache
from .mps import OneBased

__all__ = ["ProjectedExpectationCache", "init_cstorage_right", "overlap_updateleft",
           "overlap_updateright", "c_proj", "c2_proj", "project_", "projectors1",
           "projectors2"]


def overlap_updateleft(hold, A, B):
    """updateleft(hold, A, B) (mps/transfer.jl:17-20):
    hnew[c,d] = sum conj(A[a,s,c]) hold[a,b] B[b,s,d]."""
    DlA, d, DrA = A.shape
    DlB, dB, DrB = B.shape
    if d != dB or tuple(hold.shape) != (DlA, DlB):
        raise ValueError("DimensionMismatch in overlap updateleft")
    t = gemm(hold, B, (DlA, d, DrB), DlA, d * DrB, DlB)
    return gemm(A, t, (DrA, DrB), DrA, DrB, DlA * d, ta="C")


def overlap_updateright(hold, A, B):
    """updateright(hold, A, B) (mps/transfer.jl:7-10):
    hnew[c,d] = sum conj(A[c,s,b]) hold[b,e] B[d,s,e]."""
    DlA, d, DrA = A.shape
    DlB, dB, DrB = B.shape
    if d != dB or tuple(hold.shape) != (DrA, DrB):
        raise ValueError("DimensionMismatch in overlap updateright")
    t = gemm(B, hold, (DlB, d, DrA), DlB * d, DrA, DrB, tb="T")        # t[d,s,b]
    return gemm(A, t, (DlA, DlB), DlA, DlB, d * DrA, ta="R", tb="T")


def c_proj(x, cleft, cright):
    """c_proj (derivatives.jl:65-67): p[a,s,c] = cleft[a,b] x[b,s,e] cright[c,e]."""
    DlB, d, DrB = x.shape
    DlA, DrA = cleft.shape[0], cright.shape[0]
    if tuple(cleft.shape) != (DlA, DlB) or tuple(cright.shape) != (DrA, DrB):
        raise ValueError("DimensionMismatch in c_proj")
    t = gemm(cleft, x, (DlA, d, DrB), DlA, d * DrB, DlB)
    return gemm(t, cright, (DlA, d, DrA), DlA * d, DrA, DrB, tb="T")


def c2_proj(x1, x2, cleft, cright):
    """_c2_prime_2 (dmrgexcited.jl:84-86):
    p[a,s1,s2,c] = cleft[a,b] x1[b,s1,e] x2[e,s2,f] cright[c,f]."""
    DlB, d1, Dm = x1.shape
    _, d2, DrB = x2.shape
    DlA, DrA = cleft.shape[0], cright.shape[0]
    if tuple(cleft.shape) != (DlA, DlB) or tuple(cright.shape) != (DrA, DrB) or \
            x2.shape[0] != Dm:
        raise ValueError("DimensionMismatch in _c2_prime_2")
    x12 = gemm(x1, x2, (DlB, d1, d2, DrB), DlB * d1, d2 * DrB, Dm)
    t = gemm(cleft, x12, (DlA, d1, d2, DrB), DlA, d1 * d2 * DrB, DlB)
    return gemm(t, cright, (DlA, d1, d2, DrA), DlA * d1 * d2, DrA, DrB, tb="T")


def project_(y, ps):
    """_project!(y, projectors) (dmrgexcited.jl:1-6): y -= dot(y, p) p for each p
    in order, dot(y, p) = sum conj(y) p."""
    for p in ps:
        axpy(-dot(y, p), p, y)
    return y


def _eye(m, n, dtype, handle):
    e = np.zeros((m, n), dtype=dtype)
    e[np.arange(min(m, n)), np.arange(min(m, n))] = 1
    return DeviceTensor.from_numpy(e, handle, dtype)


def init_cstorage_right(psiA, psiB):
    """init_cstorage_right (finiteenv.jl:103-123): cstorage[1] = l_LL(psiA),
    cstorage[L+1] = r_RR(psiA, psiB), right updates in between."""
    L = len(psiA)
    if len(psiB) != L:
        raise ValueError("DimensionMismatch: projector length %d vs %d" % (len(psiB), L))
    if psiA[L].shape[2] != psiB[L].shape[2]:
        raise ValueError("SpaceMismatch: right boundary spaces differ")
    if psiA.dtype != psiB.dtype:
        raise TypeError("projector dtype %s vs state %s" % (psiB.dtype, psiA.dtype))
    hd = psiA.handle
    cs = OneBased([None] * (L + 1))
    cs[1] = _eye(psiA[1].shape[0], psiA[1].shape[0], psiA.dtype, hd)
    cs[L + 1] = _eye(psiA[L].shape[2], psiB[L].shape[2], psiA.dtype, hd)
    for i in range(L, 1, -1):
        cs[i] = overlap_updateright(cs[i + 1], psiA[i], psiB[i])
    return cs


class ProjectedExpectationCache(ExpectationCache):
    """struct ProjectedExpectationCache (finiteenv.jl:96-102), built by
    environments(mpo, mps, projectors) (:126-127); getproperty aliases
    state/h/env/cenvs (:129-141)."""

    def __init__(self, mpo, mps, projectors, precision="fp64"):
        super().__init__(mpo, mps, precision)
        self.projectors = list(projectors)
        self.cstorages = [init_cstorage_right(mps, p) for p in self.projectors]

    @property
    def cenvs(self):
        return self.cstorages

    def reinit_cstorages(self):
        self.cstorages = [init_cstorage_right(self.mps, p) for p in self.projectors]


def cstorage_updateleft_(env, site):
    """The overlap half of updateleft!(::ProjectedExpectationCache, site)
    (finiteenv.jl:144-149)."""
    for P, cs in zip(env.projectors, env.cstorages):
        cs[site + 1] = overlap_updateleft(cs[site], env.mps[site], P[site])


def cstorage_updateright_(env, site):
    """The overlap half of updateright!(::ProjectedExpectationCache, site)
    (finiteenv.jl:152-157)."""
    for P, cs in zip(env.projectors, env.cstorages):
        cs[site] = overlap_updateright(cs[site + 1], env.mps[site], P[site])


def projectors1(m, site):
    """[c_proj(projectors[l][site], cstorages[l][site], cstorages[l][site+1])]
    (dmrgexcited.jl:20); empty for a plain cache."""
    if not getattr(m, "projectors", None):
        return []
    return [c_proj(P[site], cs[site], cs[site + 1]) for P, cs in zip(m.projectors, m.cstorages)]


def projectors2(m, site):
    """[_c2_prime_2(projectors[l][site], projectors[l][site+1], cstorages[l][site],
    cstorages[l][site+2])] (dmrgexcited.jl:97, :125); empty for a plain cache."""
    if not getattr(m, "projectors", None):
        return []
    return [c2_proj(P[site], P[site + 1], cs[site], cs[site + 2])
            for P, cs in zip(m.projectors, m.cstorages)]
