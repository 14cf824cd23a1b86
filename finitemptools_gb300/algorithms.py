"""DMRG and TDVP drivers on device-resident tensors (algorithms/dmrg.jl,
algorithms/tdvp.jl, algorithms/dmrgexcited.jl:219-223) and expectation
values (mpo/arithmetics.jl:267-276, mpohamiltonian/arithmetics.jl:5-19,
operators/expecs.jl:29-55).

Functions ending in ``_`` mutate their first argument like the reference's
``!`` functions.  Sites are 1-based.  Every sweep keeps the MPS, the
environments and the Krylov vectors on the GPU; only scalars come back.
"""

import ctypes

import numpy as np

from ._native import C128, F64, PREC, lib
from .auxiliary import (MPSTruncation, default_truncation, dm_split, dot, gemm, leftorth, norm,
                        rightorth, scal, scale_cols, scale_rows, stable_tsvd)
from .derivatives import HeffOp
from .device import DeviceTensor, to_host_mpo
from .envs import ExpectationCache, environments, increase_bond_env_, updateleft_, updateright_
from .excited import project_, projectors1, projectors2
from .mps import max_bond_dimensions
from .transfer import updateleft, updateright
from .expansion import (DMRG1S, TDVP1S, TDVP2, dmrg1s_leftsweep_, dmrg1s_rightsweep_,
                        tdvp1s_sweep_, tdvp2_sweep_)
from .u1 import U1ExpectationCache, U1FiniteMPS, u1_expectation, u1_leftsweep_, u1_rightsweep_
from .utilities import MPOHamiltonian

__all__ = ["Defaults", "DMRG1", "DMRG2", "DMRG1S", "TDVP1", "TDVP2", "TDVP1S", "leftsweep_",
           "rightsweep_", "sweep_", "dmrg2_sweep_device_",
           "compute_", "ground_state_", "expectation", "expectation_local"]


class Defaults:
    """module Defaults (FiniteMPTools.jl:53-63)."""
    maxiter = 100
    D = 50
    tol = 1e-12
    dmrg_eig_tol = 1.0e-12
    tdvp_exp_tol = 1.0e-8
    verbosity = 1


class DMRG2:
    """@with_kw struct DMRG2 (algorithms/dmrg.jl:79-86) plus the device
    options: ``precision`` of the contractions and FP64 Krylov
    reorthogonalisation (``reorth``, not in the reference; off by default)."""

    def __init__(self, maxiter=Defaults.maxiter, tol=Defaults.tol, eig_maxiter=10,
                 eig_tol=Defaults.dmrg_eig_tol, verbosity=Defaults.verbosity, trunc=None,
                 precision="fp64", reorth=False, svd="gesvd", env_precision=None,
                 driver="python"):
        if driver not in ("python", "device"):
            raise ValueError("driver must be 'python' or 'device'")
        self.maxiter, self.tol = maxiter, tol
        self.eig_maxiter, self.eig_tol = eig_maxiter, eig_tol
        self.verbosity = verbosity
        self.trunc = trunc if trunc is not None else default_truncation()
        self.precision, self.reorth = precision, reorth
        self.svd = svd          # "gesvd" (reference semantics) or "dm" (density matrix)
        # arithmetic of the environment updates (defaults to the contractions')
        self.env_precision = env_precision or precision
        # "python": the bond loop below; "device": one fmpt_dmrg2_sweep call per sweep
        # (same library calls per bond, no Python between bonds; plain caches only)
        self.driver = driver


class DMRG1:
    """@with_kw struct DMRG1 (algorithms/dmrg.jl:8-15)."""

    def __init__(self, D=Defaults.D, maxiter=Defaults.maxiter, tol=Defaults.tol, eig_maxiter=10,
                 eig_tol=Defaults.dmrg_eig_tol, verbosity=Defaults.verbosity, precision="fp64",
                 reorth=False):
        self.D, self.maxiter, self.tol = D, maxiter, tol
        self.eig_maxiter, self.eig_tol = eig_maxiter, eig_tol
        self.verbosity = verbosity
        self.precision, self.reorth = precision, reorth


class TDVP1:
    """struct TDVP1 (algorithms/tdvp.jl:8-17); stepsize is complex for real
    time (-1j*dt).  ``krylovdim`` is the Krylov subspace of exponentiate."""

    def __init__(self, stepsize, D=Defaults.D, exptol=Defaults.tdvp_exp_tol, ishermitian=False,
                 verbosity=1, krylovdim=30, precision="fp64"):
        self.stepsize = stepsize
        self.D, self.exptol, self.ishermitian = D, exptol, ishermitian
        self.verbosity, self.krylovdim, self.precision = verbosity, krylovdim, precision


# ----------------------------------------------------------------- DMRG2
def _two_site(A, B):
    """twositemps[a,s1,s2,b] := A[a,s1,c] B[c,s2,b] (dmrg.jl:98)."""
    Dl, d1, Dm = A.shape
    _, d2, Dr = B.shape
    return gemm(A, B, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, Dm)


def _project_op(op, x, ps):
    """Projected caches (dmrgexcited.jl:96-102, :124-130): x = _project!(x, ps) in
    place (the projected tensor is the one the fidelity is measured against)
    and op composed with _project!.  No-op without projectors."""
    if ps:
        project_(x, ps)
        op.set_projectors(ps)


def _start_vector(op, A, ps):
    """One-site start vector: _project!(copy(mps[site]), p1) for projected caches
    (dmrgexcited.jl:20-23), with op composed with _project!; A itself otherwise."""
    if not ps:
        return A
    op.set_projectors(ps)
    return project_(A.copy(), ps)


def _dmrg2_bond_left(m, site, alg):
    """leftsweep! bond body (dmrg.jl:95-113): mps[site] = u, mps[site+1] = s*v."""
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    x2 = _two_site(mps[site], mps[site + 1])
    Dl, d1, d2, Dr = x2.shape
    op = HeffOp("ac2", hs[site], hs[site + 2], W1=mpo[site], W2=mpo[site + 1],
                precision=alg.precision, dtype=x2.dtype)
    _project_op(op, x2, projectors2(m, site))
    E, vecs, info, k = op.lanczos(x2, alg.eig_maxiter, alg.eig_tol, alg.reorth)
    del op
    if alg.svd == "dm":
        # U orthonormal from M M^H; s*v = U^H M, normalised with s
        u, s, svt, err = dm_split(vecs, Dl * d1, d2 * Dr, alg.trunc, 0)
        kk = s.shape[0]
        nrm = norm(s)
        scal(1.0 / nrm, s)
        scal(1.0 / nrm, svt)
    else:
        u, s, vt, err = stable_tsvd(vecs, Dl * d1, d2 * Dr, alg.trunc)
        kk = s.shape[0]
        scal(1.0 / norm(s), s)                                  # normalize!(s)
        svt = scale_rows(vt, kk, d2 * Dr, s)                    # s * v (in place)
    usv = gemm(u, svt, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, kk)
    delta = abs(1 - abs(dot(usv, x2)))   # sum x2 * conj(u s v)  (dmrg.jl:109-110)
    mps[site] = u.view_as((Dl, d1, kk))
    mps[site + 1] = svt.view_as((kk, d2, Dr))
    updateleft_(m, site)
    if alg.verbosity > 2:
        print("bond %d (left): E=%.15g lanczos k=%d info=%d D=%d" % (site, E, k, info, kk))
    return E, delta


def _grown(t, cap, dtype):
    """t itself when its buffer holds ``cap`` elements, else a copy in a buffer that does."""
    if t is not None and t.capacity >= cap * (16 if dtype == np.complex128 else 8):
        return t
    big = DeviceTensor((cap,), dtype, t.h)
    if t is not None:
        t.h.check(lib().fmpt_memcpy_d2d(t.h.ptr, big.ptr, t.ptr, t.nbytes))
    return big


def dmrg2_sweep_device_(m, alg):
    """sweep!(m, DMRG2) (dmrgexcited.jl:219-223) as ONE fmpt_dmrg2_sweep call: the
    left and right bond loops of leftsweep_/rightsweep_ run inside the library on
    the device-resident chain, with the same calls per bond (so the same Ritz
    values, tensors and environments).  Site tensors and environments are moved
    into buffers sized for the largest bonds the truncation allows, then viewed
    with their new shapes (no copy back).  Returns (energies, delta)."""
    if getattr(m, "cstorages", None) or isinstance(m, U1ExpectationCache):
        raise NotImplementedError("device sweep: plain dense ExpectationCache only")
    mps, hs = m.mps, m.hstorage
    h = mps.handle
    L = len(mps)
    dt = m.dtype
    m.precision = alg.env_precision
    phys = [mps[i].shape[1] for i in range(1, L + 1)]
    bond = [mps[1].shape[0]] + [mps[i].shape[2] for i in range(1, L + 1)]
    wb = [m.mpo[1].shape[0]] + [m.mpo[i].shape[2] for i in range(1, L + 1)]
    vmax = max_bond_dimensions(phys, alg.trunc.D)
    cb = [max(bond[b], vmax[b]) for b in range(L + 1)]
    site_cap = [cb[i] * phys[i] * cb[i + 1] for i in range(L)]
    env_cap = [cb[b] * wb[b] * cb[b] for b in range(L + 1)]
    for i in range(L):
        mps[i + 1] = _grown(mps[i + 1], site_cap[i], dt)
    for b in range(L + 1):
        hs[b + 1] = _grown(hs[b + 1], env_cap[b], dt)
    for b in range(1, L):
        mps.s[b + 1] = _grown(mps.s[b + 1] if mps.s[b + 1] is not None else
                              DeviceTensor((1,), np.float64, h), cb[b], np.float64)
    Wbufs = [to_host_mpo(W, dt) for W in m.mpo]
    arr = ctypes.c_void_p * L
    earr = ctypes.c_void_p * (L + 1)
    c_bond = (ctypes.c_int * (L + 1))(*bond)
    energies = (ctypes.c_double * max(1, 2 * L - 3))()
    delta = ctypes.c_double()
    h.check(lib().fmpt_dmrg2_sweep(
        h.ptr, C128 if dt == np.complex128 else F64, PREC[alg.precision],
        PREC[alg.env_precision], L, (ctypes.c_int * L)(*phys), c_bond,
        arr(*[mps[i + 1].ptr for i in range(L)]), (ctypes.c_int64 * L)(*site_cap),
        earr(*[hs[b + 1].ptr for b in range(L + 1)]), (ctypes.c_int64 * (L + 1))(*env_cap),
        arr(*[w.ctypes.data for w in Wbufs]), (ctypes.c_int * (L + 1))(*wb),
        earr(*([None] + [mps.s[b + 1].ptr for b in range(1, L)] + [None])),
        int(alg.trunc.D), float(alg.trunc.eps), int(alg.eig_maxiter), float(alg.eig_tol),
        1 if alg.reorth else 0, 1 if alg.svd == "dm" else 0, energies, ctypes.byref(delta)))
    bond = list(c_bond)
    for i in range(L):
        mps[i + 1].view_as((bond[i], phys[i], bond[i + 1]))
    for b in range(L + 1):
        hs[b + 1].view_as((bond[b], wb[b], bond[b]))
    for b in range(1, L):
        mps.s[b + 1].view_as((bond[b],))
    return list(energies)[:2 * L - 3], delta.value


def leftsweep_(m, alg):
    """leftsweep!(m, alg) for DMRG2 (dmrg.jl:89-115) and DMRG1 (:27-52)."""
    if isinstance(m, U1ExpectationCache):
        if not isinstance(alg, DMRG2):
            raise NotImplementedError("U(1) tensors: DMRG2 sweeps only")
        return u1_leftsweep_(m, alg)
    if isinstance(alg, DMRG1S):
        return dmrg1s_leftsweep_(m, alg)
    if isinstance(alg, DMRG1):
        return _dmrg1_leftsweep(m, alg)
    m.precision = alg.env_precision
    Es, delta = [], 0.0
    for site in range(1, len(m.mps) - 1):
        E, dl = _dmrg2_bond_left(m, site, alg)
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta


def rightsweep_(m, alg):
    """rightsweep!(m, alg) for DMRG2 (dmrg.jl:117-144) and DMRG1 (:54-76)."""
    if isinstance(m, U1ExpectationCache):
        if not isinstance(alg, DMRG2):
            raise NotImplementedError("U(1) tensors: DMRG2 sweeps only")
        return u1_rightsweep_(m, alg)
    if isinstance(alg, DMRG1S):
        return dmrg1s_rightsweep_(m, alg)
    if isinstance(alg, DMRG1):
        return _dmrg1_rightsweep(m, alg)
    m.precision = alg.env_precision
    Es, delta = [], 0.0
    for site in range(len(m.mps) - 1, 0, -1):
        E, dl = _dmrg2_bond_right(m, site, alg)
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta


def _dmrg2_bond_right(m, site, alg):
    """rightsweep! bond body (dmrg.jl:123-142): mps[site] = u*s,
    mps[site+1] = v, mps.s[site+1] = s."""
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    x2 = _two_site(mps[site], mps[site + 1])
    Dl, d1, d2, Dr = x2.shape
    op = HeffOp("ac2", hs[site], hs[site + 2], W1=mpo[site], W2=mpo[site + 1],
                precision=alg.precision, dtype=x2.dtype)
    _project_op(op, x2, projectors2(m, site))
    E, vecs, info, k = op.lanczos(x2, alg.eig_maxiter, alg.eig_tol, alg.reorth)
    del op
    if alg.svd == "dm":
        # v^H orthonormal from M^H M; u*s = M V, normalised with s
        us, s, vt, err = dm_split(vecs, Dl * d1, d2 * Dr, alg.trunc, 1)
        kk = s.shape[0]
        nrm = norm(s)
        scal(1.0 / nrm, s)
        scal(1.0 / nrm, us)
        usv = gemm(us, vt, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, kk)
        delta = abs(1 - abs(dot(usv, x2)))
        del usv
    else:
        u, s, vt, err = stable_tsvd(vecs, Dl * d1, d2 * Dr, alg.trunc)
        kk = s.shape[0]
        scal(1.0 / norm(s), s)
        # fidelity first (needs u, s, v before they are absorbed)
        svt = scale_rows(vt.copy(), kk, d2 * Dr, s)
        usv = gemm(u, svt, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, kk)
        delta = abs(1 - abs(dot(usv, x2)))
        del svt, usv
        us = scale_cols(u, Dl * d1, kk, s)
    mps[site] = us.view_as((Dl, d1, kk))
    mps[site + 1] = vt.view_as((kk, d2, Dr))
    mps.s[site + 1] = s
    updateright_(m, site + 1)
    if alg.verbosity > 2:
        print("bond %d (right): E=%.15g lanczos k=%d D=%d" % (site, E, k, kk))
    return E, delta


# ----------------------------------------------------------------- DMRG1
def _galerkin(m, site, precision):
    """calc_galerkin (dmrg.jl:17-24): || leftnull(A)^H * ac_prime(A) ||, zero when
    the left null space is empty.  leftnull spans the complement of the thin
    QR factor Q of A, so the norm is ||y - Q Q^H y||."""
    A = m.mps[site]
    Dl, d, Dr = A.shape
    if Dl * d <= Dr:
        return 0.0
    op = HeffOp("ac", m.hstorage[site], m.hstorage[site + 1], W1=m.mpo[site],
                precision=precision, dtype=A.dtype)
    y = op(A)
    Q, _ = leftorth(A, Dl * d, Dr)
    r = Q.shape[1]
    # y - Q (Q^H y)
    qy = gemm(Q, y, (r, Dr), r, Dr, Dl * d, ta="C")
    gemm(Q, qy, None, Dl * d, Dr, r, alpha=-1.0, beta=1.0, C=y)
    return norm(y)


def _dmrg1_leftsweep(m, alg):
    increase_bond_env_(m, alg.D)
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    Es, delta = [], 0.0
    for site in range(1, len(mps)):
        A = mps[site]
        op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                    dtype=A.dtype)
        x0 = _start_vector(op, A, projectors1(m, site))
        E, vec, _, _ = op.lanczos(x0, alg.eig_maxiter, alg.eig_tol, alg.reorth)
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


def _dmrg1_rightsweep(m, alg):
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    Es, delta = [], 0.0
    for site in range(len(mps), 1, -1):
        A = mps[site]
        op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                    dtype=A.dtype)
        x0 = _start_vector(op, A, projectors1(m, site))
        E, vec, _, _ = op.lanczos(x0, alg.eig_maxiter, alg.eig_tol, alg.reorth)
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


# ----------------------------------------------------------------- TDVP1
def _env_prec(alg, A):
    """Arithmetic of TDVP1's environment updates: the contractions' precision for
    real data; FP64 for complex data (the tensor-core environment update is real
    only, and at the TDVP bond dimensions it is a small share of a step)."""
    return "fp64" if A.dtype == np.complex128 else alg.precision


def _tdvp1_leftsweep(m, alg):
    """_leftsweep!(m, ::TDVP1) (tdvp.jl:19-44)."""
    increase_bond_env_(m, alg.D)
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    dt = alg.stepsize
    L = len(mps)
    for site in range(1, L):
        A = mps[site]
        op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                    dtype=A.dtype)
        tmp = op.exponentiate(dt / 2, A, alg.exptol / abs(dt / 2), alg.krylovdim)
        del op
        Dl, d, Dr = A.shape
        Q, v = leftorth(tmp, Dl * d, Dr)
        r = Q.shape[1]
        mps[site] = Q.view_as((Dl, d, r))
        hnew = updateleft(hs[site], mps[site], mpo[site], mps[site], _env_prec(alg, A))
        opc = HeffOp("c", hnew, hs[site + 1], precision=alg.precision, dtype=A.dtype)
        v = opc.exponentiate(-dt / 2, v, alg.exptol / abs(dt / 2), alg.krylovdim)
        del opc
        B = mps[site + 1]
        mps[site + 1] = gemm(v, B, (r, B.shape[1], B.shape[2]), r, B.shape[1] * B.shape[2], Dr)
        hs[site + 1] = hnew
    site = L
    op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                dtype=mps[site].dtype)
    mps[site] = op.exponentiate(dt, mps[site], alg.exptol / abs(dt), alg.krylovdim)


def _tdvp1_rightsweep(m, alg):
    """_rightsweep!(m, ::TDVP1) (tdvp.jl:46-69)."""
    mps, mpo, hs = m.mps, m.mpo, m.hstorage
    dt = alg.stepsize
    L = len(mps)
    for site in range(L - 1, 0, -1):
        B = mps[site + 1]
        Dl, d, Dr = B.shape
        v, Q = rightorth(B, Dl, d * Dr)
        r = Q.shape[0]
        mps[site + 1] = Q.view_as((r, d, Dr))
        hnew = updateright(hs[site + 2], mps[site + 1], mpo[site + 1], mps[site + 1],
                           _env_prec(alg, B))
        opc = HeffOp("c", hs[site + 1], hnew, precision=alg.precision, dtype=B.dtype)
        v = opc.exponentiate(-dt / 2, v, alg.exptol / abs(dt / 2), alg.krylovdim)
        del opc
        hs[site + 1] = hnew
        P = mps[site]
        mps[site] = gemm(P, v, (P.shape[0], P.shape[1], r), P.shape[0] * P.shape[1], r, Dl)
        op = HeffOp("ac", hs[site], hs[site + 1], W1=mpo[site], precision=alg.precision,
                    dtype=P.dtype)
        mps[site] = op.exponentiate(dt / 2, mps[site], alg.exptol / abs(dt / 2), alg.krylovdim)


# --------------------------------------------------------------- drivers
def sweep_(m, alg):
    """sweep!(m, alg): DMRG returns (Energies, delta) (dmrgexcited.jl:219-223);
    TDVP evolves in place (tdvp.jl:219-222)."""
    if isinstance(alg, TDVP1):
        _tdvp1_leftsweep(m, alg)
        _tdvp1_rightsweep(m, alg)
        return None
    if isinstance(alg, TDVP2):
        tdvp2_sweep_(m, alg)
        return None
    if isinstance(alg, TDVP1S):
        tdvp1s_sweep_(m, alg)
        return None
    if isinstance(alg, DMRG2) and alg.driver == "device":
        return dmrg2_sweep_device_(m, alg)
    E1, d1 = leftsweep_(m, alg)
    E2, d2 = rightsweep_(m, alg)
    return E1 + E2, max(d1, d2)


def compute_(env, alg):
    """compute!(env, alg) (dmrg.jl:221-234)."""
    all_E = []
    it = 0
    delta = 2 * alg.tol
    while it < alg.maxiter and delta > alg.tol:
        Es, delta = sweep_(env, alg)
        all_E.extend(Es)
        it += 1
    return all_E, delta


def ground_state_(state, h, alg=None):
    """ground_state!(state, h, alg=DMRG1S()) (dmrg.jl:240)."""
    alg = alg if alg is not None else DMRG1S()
    if isinstance(state, U1FiniteMPS):
        return compute_(U1ExpectationCache(h, state), alg)
    return compute_(environments(h, state, alg.precision), alg)


# ------------------------------------------------------------ observables
def expectation(psiA, h, psiB=None, precision="fp64"):
    """expectation(psiA, h::FiniteMPO | MPOHamiltonian, psiB): a chain of
    updateright from r_RR, closed with l_LL."""
    if isinstance(psiA, U1FiniteMPS):
        if psiB is not None and psiB is not psiA:
            raise NotImplementedError("U(1) expectation: <psi|H|psi> only")
        return u1_expectation(psiA, h)
    psiB = psiA if psiB is None else psiB
    L = len(psiA)
    if isinstance(h, MPOHamiltonian):
        Ws = h.site_tensors(L)
    else:
        Ws = list(h)
    dt = np.complex128 if (psiA.dtype == np.complex128 or psiB.dtype == np.complex128 or
                           any(np.iscomplexobj(W) for W in Ws)) else np.float64
    w = Ws[-1].shape[2]
    e = np.zeros((1, w, 1), dtype=dt)
    e[0, w - 1, 0] = 1
    hold = DeviceTensor.from_numpy(e, psiA.handle, dt)
    for i in range(L, 0, -1):
        hold = updateright(hold, psiA[i], Ws[i - 1].astype(dt), psiB[i], precision)
    v = hold.numpy().reshape(-1)
    return v[0]


def expectation_local(psi, site, op):
    """<psi|O_site|psi>/<psi|psi> for a one-site operator, by overlap chains
    (operators/expecs.jl:29-55 with a one-site QTerm)."""
    L = len(psi)
    d = psi[1].shape[1]
    dt = np.complex128 if (psi.dtype == np.complex128 or np.iscomplexobj(op)) else np.float64
    one = np.ones((1, 1, 1), dtype=dt)
    hold = DeviceTensor.from_numpy(one, psi.handle, dt)
    nrm = DeviceTensor.from_numpy(one, psi.handle, dt)
    I = np.eye(d, dtype=dt).reshape(1, d, 1, d)
    O = np.asarray(op, dtype=dt).reshape(1, d, 1, d)
    for i in range(L, 0, -1):
        hold = updateright(hold, psi[i], O if i == site else I, psi[i])
        nrm = updateright(nrm, psi[i], None, psi[i])
    return hold.numpy().reshape(-1)[0] / nrm.numpy().reshape(-1)[0]
