"""Sweep-level algorithms of the reference restated in numpy (test infrastructure only).

An MPS is a plain list of numpy site tensors A[a, s, b]; an MPO is a list of
dense W[wl, s_out, wr, s_in] (a Schur-form MPOHamiltonian is passed as its
dense embedding plus ``schur=True`` environments).  Environments follow
envs/finiteenv.jl: ``hstorage[i]`` (0-based list of length L+1) is the left
environment of site i for i <= centre and the right environment of site i-1
beyond it.
"""

import numpy as np

from .core import (ac_prime, ac2_prime, c_prime, updateleft, updateright,
                   l_LL_dense, r_RR_dense, l_LL_schur, r_RR_schur,
                   simple_lanczos_solver, stable_tsvd, MPSTruncation,
                   leftorth_qr, rightorth_lq, krylov_exponentiate)

__all__ = [
    "max_virtual_dims", "randommps", "prodmps", "canonicalize", "increase_bond",
    "bond_dimension", "OracleEnv", "environments", "dmrg2_leftsweep",
    "dmrg2_rightsweep", "dmrg2_sweep", "dmrg1_leftsweep", "dmrg1_rightsweep",
    "dmrg1_sweep", "tdvp1_sweep", "expectation_mpo", "mps_to_dense",
    "mpo_to_dense", "single_site_expectation",
]


# ------------------------------------------------------------------ states
def max_virtual_dims(ds, D):
    """Virtual dimensions of FiniteMPS(f, T, physpaces, C^D)
    (mps/initializers.jl:15-27) == max_bond_dimensions(physpaces::Vector{Int}, D)
    (mps/finitemps.jl:283-297)."""
    L = len(ds)
    v = [1] * (L + 1)
    for i in range(1, L):
        v[i] = min(v[i - 1] * ds[i - 1], D)
    v[L] = 1
    for i in range(L - 1, 0, -1):
        v[i] = min(v[i], ds[i] * v[i + 1])
    return v


def randommps(L, d, D, rng, dtype=np.float64):
    """randommps(T, L; d, D) (mps/initializers.jl:101-108): iid N(0,1) site
    tensors on the maximal virtual spaces capped at D.  Entries are drawn in
    column-major order per site from ``rng`` (numpy Generator); complex
    entries draw the real then the imaginary plane."""
    v = max_virtual_dims([d] * L, D)
    out = []
    for i in range(L):
        shape = (v[i], d, v[i + 1])
        n = int(np.prod(shape))
        if np.issubdtype(dtype, np.complexfloating):
            re = rng.standard_normal(n)
            im = rng.standard_normal(n)
            flat = (re + 1j * im) / np.sqrt(2.0)
        else:
            flat = rng.standard_normal(n)
        out.append(flat.reshape(shape, order="F").astype(dtype))
    return out


def prodmps(vectors, dtype=np.float64):
    """prodmps(physectors::Vector{Vector}) (mps/initializers.jl:80-87)."""
    return [np.asarray(v, dtype=dtype).reshape(1, len(v), 1) for v in vectors]


def bond_dimension(mps):
    return max(A.shape[2] for A in mps[:-1])


def canonicalize(mps, normalize=False):
    """right_canonicalize! (mps/orth.jl:40-49): SVD leftorth! sweep, optional
    normalisation of the last site, SVD rightorth! sweep, no truncation.
    Returns (mps, svectors) with svectors[i] the singular values on bond i."""
    L = len(mps)
    mps = [A.copy() for A in mps]
    svals = [None] * (L + 1)
    for i in range(L - 1):                                   # orth.jl:5-20
        Dl, d, Dr = mps[i].shape
        u, s, vh, _ = stable_tsvd(mps[i].reshape(Dl * d, Dr, order="F"))
        mps[i] = u.reshape(Dl, d, u.shape[1], order="F")
        v2 = s[:, None] * vh
        mps[i + 1] = np.tensordot(v2, mps[i + 1], axes=([1], [0]))
        svals[i + 1] = s
    if normalize:
        mps[-1] = mps[-1] / np.linalg.norm(mps[-1])
    for i in range(L - 1, 0, -1):                            # orth.jl:22-37
        Dl, d, Dr = mps[i].shape
        u, s, vh, _ = stable_tsvd(mps[i].reshape(Dl, d * Dr, order="F"))
        mps[i] = vh.reshape(vh.shape[0], d, Dr, order="F")
        u2 = u * s[None, :]
        mps[i - 1] = np.tensordot(mps[i - 1], u2, axes=([2], [0]))
        svals[i] = s
    return mps, svals


def increase_bond(mps, D):
    """increase_bond!(psi::FiniteNonSymmetricMPS; D) (mps/finitemps.jl:302-317):
    zero-pad every site tensor to the capped maximal virtual dimensions."""
    if bond_dimension(mps) >= D:
        return mps
    ds = [A.shape[1] for A in mps]
    v = max_virtual_dims(ds, D)
    out = []
    for i, A in enumerate(mps):
        sl = max(min(v[i], D), A.shape[0])
        sr = max(min(v[i + 1], D), A.shape[2])
        m = np.zeros((sl, A.shape[1], sr), dtype=A.dtype)
        m[:A.shape[0], :, :A.shape[2]] = A
        out.append(m)
    return out


# ------------------------------------------------------------ environments
class OracleEnv:
    """ExpectationCache (envs/finiteenv.jl:51-78)."""

    def __init__(self, mpo, mps, schur=False):
        self.mpo = mpo
        self.mps = [A.copy() for A in mps]
        self.schur = schur
        self.hstorage = None
        self.init_hstorage(center=1)

    def boundaries(self):
        T = np.result_type(self.mps[0], self.mpo[0])
        if self.schur:
            return l_LL_schur(self.mpo[0].shape[0], T), r_RR_schur(self.mpo[-1].shape[2], T)
        return l_LL_dense(T), r_RR_dense(T)

    def init_hstorage(self, center=1):
        """init_hstorage! (envs/finiteenv.jl:1-21), 1-based centre."""
        L = len(self.mps)
        hs = [None] * (L + 1)
        hs[0], hs[L] = self.boundaries()
        for i in range(L, center, -1):           # Julia i in L:-1:center+1
            hs[i - 1] = updateright(hs[i], self.mps[i - 1], self.mpo[i - 1], self.mps[i - 1])
        for i in range(1, center):               # Julia i in 1:center-1
            hs[i] = updateleft(hs[i - 1], self.mps[i - 1], self.mpo[i - 1], self.mps[i - 1])
        self.hstorage = hs

    # 1-based site numbering as in the reference
    def updateleft_(self, site):
        """updateleft!(env, site): hstorage[site+1] = updateleft(hstorage[site], ...)"""
        self.hstorage[site] = updateleft(self.hstorage[site - 1], self.mps[site - 1],
                                         self.mpo[site - 1], self.mps[site - 1])

    def updateright_(self, site):
        """updateright!(env, site): hstorage[site] = updateright(hstorage[site+1], ...)"""
        self.hstorage[site - 1] = updateright(self.hstorage[site], self.mps[site - 1],
                                              self.mpo[site - 1], self.mps[site - 1])

    def increase_bond_(self, D):
        """increase_bond!(m::ExpectationCache; D) (envs/finiteenv.jl:87-93)."""
        if bond_dimension(self.mps) < D:
            self.mps = increase_bond(self.mps, D)
            self.mps, _ = canonicalize(self.mps, normalize=False)
            self.init_hstorage(center=1)


def environments(mpo, mps, schur=False):
    return OracleEnv(mpo, mps, schur=schur)


# ------------------------------------------------------------------- DMRG2
def _dmrg2_bond(env, site, trunc, eig_maxiter, eig_tol, direction):
    """Body of leftsweep!/rightsweep!(::DMRG2) for one bond (algorithms/dmrg.jl:95-113,
    :123-142); ``site`` is 1-based."""
    mps, mpo, hs = env.mps, env.mpo, env.hstorage
    A, B = mps[site - 1], mps[site]
    x2 = np.tensordot(A, B, axes=([2], [0]))                       # dmrg.jl:98
    shape = x2.shape
    W1, W2, L, R = mpo[site - 1], mpo[site], hs[site - 1], hs[site + 1]

    def f(v):
        return ac2_prime(v.reshape(shape, order="F"), W1, W2, L, R).ravel(order="F")

    E, vec, info, k = simple_lanczos_solver(f, x2.ravel(order="F"), eig_maxiter, eig_tol)
    vec = vec.reshape(shape, order="F")
    Dl, d1, d2, Dr = shape
    u, s, vh, err = stable_tsvd(vec.reshape(Dl * d1, d2 * Dr, order="F"), trunc)
    s = s / np.linalg.norm(s)                                      # normalize!(s)
    U = u.reshape(Dl, d1, u.shape[1], order="F")
    V = vh.reshape(vh.shape[0], d2, Dr, order="F")
    usv = np.tensordot(U * s[None, None, :], V, axes=([2], [0]))
    err_1 = np.vdot(usv, x2)            # sum x2 * conj(u s v)   (dmrg.jl:109)
    delta = abs(1 - abs(err_1))
    if direction == "left":
        mps[site - 1] = U
        mps[site] = s[:, None, None] * V
        env.updateleft_(site)
    else:
        mps[site - 1] = U * s[None, None, :]
        mps[site] = V
        env.updateright_(site + 1)
    return E, delta, k


def dmrg2_leftsweep(env, trunc, eig_maxiter=10, eig_tol=1e-12):
    """leftsweep!(m, ::DMRG2) (algorithms/dmrg.jl:89-115): bonds 1..L-2."""
    Es, delta = [], 0.0
    for site in range(1, len(env.mps) - 1):
        E, dl, _ = _dmrg2_bond(env, site, trunc, eig_maxiter, eig_tol, "left")
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta


def dmrg2_rightsweep(env, trunc, eig_maxiter=10, eig_tol=1e-12):
    """rightsweep!(m, ::DMRG2) (algorithms/dmrg.jl:117-144): bonds L-1..1."""
    Es, delta = [], 0.0
    for site in range(len(env.mps) - 1, 0, -1):
        E, dl, _ = _dmrg2_bond(env, site, trunc, eig_maxiter, eig_tol, "right")
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta


def dmrg2_sweep(env, trunc=None, eig_maxiter=10, eig_tol=1e-12):
    """sweep!(m, ::DMRG2) (algorithms/dmrgexcited.jl:219-223)."""
    trunc = trunc or MPSTruncation(100, 1e-8)
    E1, d1 = dmrg2_leftsweep(env, trunc, eig_maxiter, eig_tol)
    E2, d2 = dmrg2_rightsweep(env, trunc, eig_maxiter, eig_tol)
    return E1 + E2, max(d1, d2)


# ------------------------------------------------------------------- DMRG1
def _galerkin(env, site, vec):
    """calc_galerkin (algorithms/dmrg.jl:17-24) on the optimised tensor: the
    norm of the part of H_eff*A orthogonal to A's left span."""
    mps, mpo, hs = env.mps, env.mpo, env.hstorage
    A = mps[site - 1]
    y = ac_prime(A, mpo[site - 1], hs[site - 1], hs[site])
    Dl, d, Dr = A.shape
    M = A.reshape(Dl * d, Dr, order="F")
    Y = y.reshape(Dl * d, Dr, order="F")
    if M.shape[0] <= M.shape[1]:
        return 0.0                      # leftnull is empty: norm of an empty map
    Q, _ = np.linalg.qr(M, mode="complete")
    N = Q[:, M.shape[1]:]
    return float(np.linalg.norm(N.conj().T @ Y))


def dmrg1_leftsweep(env, D, eig_maxiter=10, eig_tol=1e-12):
    """leftsweep!(m, ::DMRG1) (algorithms/dmrg.jl:27-52)."""
    env.increase_bond_(D)
    Es, delta = [], 0.0
    for site in range(1, len(env.mps)):
        mps, mpo, hs = env.mps, env.mpo, env.hstorage
        A = mps[site - 1]
        W, L, R = mpo[site - 1], hs[site - 1], hs[site]
        E, vec, _, _ = simple_lanczos_solver(
            lambda v: ac_prime(v.reshape(A.shape, order="F"), W, L, R).ravel(order="F"),
            A.ravel(order="F"), eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, _galerkin(env, site, A))
        Q, Rm = leftorth_qr(vec.reshape(A.shape, order="F"))
        mps[site - 1] = Q
        mps[site] = np.tensordot(Rm, mps[site], axes=([1], [0]))
        env.updateleft_(site)
    return Es, delta


def dmrg1_rightsweep(env, eig_maxiter=10, eig_tol=1e-12):
    """rightsweep!(m, ::DMRG1) (algorithms/dmrg.jl:54-76)."""
    Es, delta = [], 0.0
    for site in range(len(env.mps), 1, -1):
        mps, mpo, hs = env.mps, env.mpo, env.hstorage
        A = mps[site - 1]
        W, L, R = mpo[site - 1], hs[site - 1], hs[site]
        E, vec, _, _ = simple_lanczos_solver(
            lambda v: ac_prime(v.reshape(A.shape, order="F"), W, L, R).ravel(order="F"),
            A.ravel(order="F"), eig_maxiter, eig_tol)
        Es.append(E)
        delta = max(delta, _galerkin(env, site, A))
        Lm, Q = rightorth_lq(vec.reshape(A.shape, order="F"))
        mps[site - 1] = Q
        mps[site - 2] = np.tensordot(mps[site - 2], Lm, axes=([2], [0]))
        env.updateright_(site)
    return Es, delta


def dmrg1_sweep(env, D=50, eig_maxiter=10, eig_tol=1e-12):
    E1, d1 = dmrg1_leftsweep(env, D, eig_maxiter, eig_tol)
    E2, d2 = dmrg1_rightsweep(env, eig_maxiter, eig_tol)
    return E1 + E2, max(d1, d2)


# ------------------------------------------------------------------- TDVP1
def tdvp1_sweep(env, dt, D=50, exptol=1e-8, krylovdim=30):
    """sweep!(m, ::TDVP1) = _leftsweep! + _rightsweep! (algorithms/tdvp.jl:19-69,
    219-222).  ``dt`` is the reference's stepsize (real time: -1j*dt)."""
    env.increase_bond_(D)                                          # tdvp.jl:20
    mps, mpo, hs = env.mps, env.mpo, env.hstorage
    L = len(mps)

    def expo(f, t, x):
        shape = x.shape
        y = krylov_exponentiate(lambda v: f(v.reshape(shape, order="F")).ravel(order="F"),
                                t, x.ravel(order="F"), tol=exptol, krylovdim=krylovdim)
        return y.reshape(shape, order="F")

    for site in range(1, L):                                       # tdvp.jl:28-40
        W, Le, Re = mpo[site - 1], hs[site - 1], hs[site]
        tmp = expo(lambda x: ac_prime(x, W, Le, Re), dt / 2, mps[site - 1])
        Q, v = leftorth_qr(tmp)
        mps[site - 1] = Q
        hnew = updateleft(hs[site - 1], Q, W, Q)
        v = expo(lambda x: c_prime(x, hnew, Re), -dt / 2, v)
        mps[site] = np.tensordot(v, mps[site], axes=([1], [0]))
        hs[site] = hnew
    site = L                                                       # tdvp.jl:41-43
    mps[site - 1] = expo(lambda x: ac_prime(x, mpo[site - 1], hs[site - 1], hs[site]), dt,
                         mps[site - 1])
    for site in range(L - 1, 0, -1):                               # tdvp.jl:53-68
        v, Q = rightorth_lq(mps[site])
        mps[site] = Q
        hnew = updateright(hs[site + 1], Q, mpo[site], Q)
        Le = hs[site]
        v = expo(lambda x: c_prime(x, Le, hnew), -dt / 2, v)
        hs[site] = hnew
        mps[site - 1] = np.tensordot(mps[site - 1], v, axes=([2], [0]))
        W, Le2, Re2 = mpo[site - 1], hs[site - 1], hs[site]
        mps[site - 1] = expo(lambda x: ac_prime(x, W, Le2, Re2), dt / 2, mps[site - 1])


# ----------------------------------------------------------- observables
def expectation_mpo(mps, mpo, schur=False):
    """expectation(psi, h::FiniteMPO, psi) (mpo/arithmetics.jl:267-276) and the
    MPOHamiltonian variant (mpohamiltonian/arithmetics.jl:5-19)."""
    T = np.result_type(mps[0], mpo[0])
    if schur:
        hold = r_RR_schur(mpo[-1].shape[2], T)
    else:
        hold = r_RR_dense(T)
    for i in range(len(mps) - 1, -1, -1):
        hold = updateright(hold, mps[i], mpo[i], mps[i])
    if schur:
        left = l_LL_schur(mpo[0].shape[0], T)
        return np.sum(left * hold)
    return hold.reshape(-1)[0]


def single_site_expectation(mps, site, op):
    """<psi|O_site|psi> / <psi|psi> by an overlap chain (operators/expecs.jl:29-55
    with a one-site QTerm).  ``site`` is 1-based."""
    T = np.result_type(mps[0], op)
    hold = np.ones((1, 1, 1), dtype=T)
    norm = np.ones((1, 1, 1), dtype=T)
    for i in range(len(mps) - 1, -1, -1):
        A = mps[i]
        W = (op if i == site - 1 else np.eye(A.shape[1], dtype=T)).reshape(1, A.shape[1], 1, A.shape[1])
        hold = updateright(hold, A, W, A)
        norm = updateright(norm, A, np.eye(A.shape[1], dtype=T).reshape(1, A.shape[1], 1, A.shape[1]), A)
    return hold.reshape(-1)[0] / norm.reshape(-1)[0]


def mps_to_dense(mps):
    """Full state vector (column-major over sites: site 1 fastest, like a
    Julia reshape of the contracted chain)."""
    psi = mps[0]                          # [1, d, D]
    for A in mps[1:]:
        psi = np.tensordot(psi, A, axes=([psi.ndim - 1], [0]))
    return psi.reshape(-1, order="F")


def mpo_to_dense(mpo):
    """Dense operator matrix (same site ordering as mps_to_dense)."""
    T = mpo[0]                            # [1, s', w, s]
    op = np.transpose(T, (0, 2, 1, 3))    # [wl, wr, s', s]
    op = op[0]                            # [wr, s', s]
    n = op.shape[1]
    op = np.transpose(op, (1, 2, 0))      # [s', s, wr]
    for W in mpo[1:]:
        d = W.shape[1]
        # op[(out), (in), w] x W[w, s', w2, s]
        t = np.tensordot(op, W, axes=([2], [0]))   # [out, in, s', w2, s]
        t = np.transpose(t, (0, 2, 1, 4, 3))        # [out, s', in, s, w2]
        n = n * d
        op = t.reshape(n, n, W.shape[2], order="F")
    return op[:, :, 0]
