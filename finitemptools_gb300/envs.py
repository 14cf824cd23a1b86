"""ExpectationCache: device-resident environment storage (envs/finiteenv.jl).

``hstorage[i]`` (1-based, length L+1) is the left environment of site i for
i <= centre and the right environment of site i-1 beyond it, as in
init_hstorage! (finiteenv.jl:1-21).
"""

import numpy as np

from .device import DeviceTensor
from .mps import OneBased, bond_dimension, canonicalize_, increase_bond_
from .transfer import updateleft, updateright
from .utilities import MPOHamiltonian

__all__ = ["ExpectationCache", "environments", "updateleft_", "updateright_",
           "init_hstorage_", "l_LL", "r_RR"]


def _mpo_tensors(mpo, L):
    """Dense site tensors and whether the Schur boundary vectors apply."""
    if isinstance(mpo, MPOHamiltonian):
        return [np.asarray(W) for W in mpo.site_tensors(L)], True
    Ws = [np.asarray(W) for W in mpo]
    if len(Ws) != L:
        raise ValueError("DimensionMismatch: MPO length %d vs MPS length %d" % (len(Ws), L))
    if Ws[0].shape[0] != 1 or Ws[-1].shape[2] != 1:
        raise ValueError("operator must be strict.")
    return Ws, False


def l_LL(w, dtype, handle, schur):
    """Left boundary: 1x1x1 identity for a FiniteMPO (mpo/arithmetics.jl:258),
    ones at w=1 for an MPOHamiltonian (mpohamiltonian/transfer.jl:26-44)."""
    e = np.zeros((1, w, 1), dtype=dtype)
    e[0, 0, 0] = 1
    return DeviceTensor.from_numpy(e, handle, dtype)


def r_RR(w, dtype, handle, schur):
    """Right boundary: ones at w=last (mpohamiltonian/transfer.jl:3-23)."""
    e = np.zeros((1, w, 1), dtype=dtype)
    e[0, w - 1, 0] = 1
    return DeviceTensor.from_numpy(e, handle, dtype)


class ExpectationCache:
    """struct ExpectationCache (finiteenv.jl:51-55) with the getproperty
    aliases state/h/env (:59-69)."""

    def __init__(self, mpo, mps, precision="fp64"):
        self.h_input = mpo
        L = len(mps)
        Ws, schur = _mpo_tensors(mpo, L)
        cplx = mps.dtype == np.complex128 or any(np.iscomplexobj(W) for W in Ws)
        self.dtype = np.dtype(np.complex128 if cplx else np.float64)
        self.mpo = OneBased([W.astype(self.dtype) for W in Ws])
        self.mps = mps
        self.schur = schur
        self.precision = precision
        self.hstorage = OneBased([None] * (L + 1))
        init_hstorage_(self, center=1)

    # getproperty aliases
    @property
    def state(self):
        return self.mps

    @property
    def h(self):
        return self.mpo

    @property
    def env(self):
        return self.hstorage


def init_hstorage_(m, center=1):
    """init_hstorage! (finiteenv.jl:1-21)."""
    L = len(m.mps)
    hd = m.mps.handle
    hs = m.hstorage
    hs[L + 1] = r_RR(m.mpo[L].shape[2], m.dtype, hd, m.schur)
    hs[1] = l_LL(m.mpo[1].shape[0], m.dtype, hd, m.schur)
    for i in range(L, center, -1):
        hs[i] = updateright(hs[i + 1], m.mps[i], m.mpo[i], m.mps[i], m.precision)
    for i in range(1, center):
        hs[i + 1] = updateleft(hs[i], m.mps[i], m.mpo[i], m.mps[i], m.precision)
    return hs


def environments(mpo, mps, projectors=None, precision="fp64"):
    """environments(mpo, mps) (finiteenv.jl:57), and environments(mpo, mps,
    projectors) (:126-127), which returns a ProjectedExpectationCache for
    excited-state sweeps.  A string in the third position is the precision."""
    if isinstance(projectors, str):
        projectors, precision = None, projectors
    if mps.dtype != np.complex128 and any(np.iscomplexobj(W) for W in
                                          (mpo.site_tensors(len(mps)) if isinstance(mpo, MPOHamiltonian) else mpo)):
        raise TypeError("complex MPO needs a complex MPS")
    if projectors is not None:
        from .excited import ProjectedExpectationCache
        return ProjectedExpectationCache(mpo, mps, projectors, precision)
    return ExpectationCache(mpo, mps, precision)


def updateleft_(env, site):
    """updateleft!(env, site) (finiteenv.jl:72-74); a projected cache also
    updates its overlap storages (:144-149)."""
    env.hstorage[site + 1] = updateleft(env.hstorage[site], env.mps[site], env.mpo[site],
                                        env.mps[site], env.precision)
    if getattr(env, "cstorages", None):
        from .excited import cstorage_updateleft_
        cstorage_updateleft_(env, site)


def updateright_(env, site):
    """updateright!(env, site) (finiteenv.jl:76-78); a projected cache also
    updates its overlap storages (:152-157)."""
    env.hstorage[site] = updateright(env.hstorage[site + 1], env.mps[site], env.mpo[site],
                                     env.mps[site], env.precision)
    if getattr(env, "cstorages", None):
        from .excited import cstorage_updateright_
        cstorage_updateright_(env, site)


def increase_bond_env_(env, D):
    """increase_bond!(m::ExpectationCache; D) (finiteenv.jl:87-93) and
    (m::ProjectedExpectationCache; D) (:159-168)."""
    if bond_dimension(env.mps) < D:
        increase_bond_(env.mps, D)
        canonicalize_(env.mps, normalize=False)
        init_hstorage_(env, 1)
        if getattr(env, "cstorages", None):
            env.reinit_cstorages()
