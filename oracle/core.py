"""Local kernels of the reference restated in numpy (test infrastructure only).

Index conventions (mps/abstractdefs.jl:4, mpo/abstractdefs.jl:4):
  MPS site tensor   A[a, s, b]            (left virtual, physical, right virtual)
  MPO site tensor   W[wl, s_out, wr, s_in]
  left environment  L[a', w, a]           (bra, mpo, ket)
  right environment R[b', w, b]           (bra, mpo, ket)
  two-site tensor   x2[a, s1, s2, b]
The pairwise contraction order of every ``@tensor`` is kept (TensorOperations
contracts left to right), so the CPU timing of these functions is the
reference's own arithmetic: permute + BLAS gemm per pair.
"""

import numpy as np
import scipy.linalg

__all__ = [
    "ac_prime", "ac2_prime", "c_prime", "ac2_prime_schur", "ac_prime_schur",
    "c_prime_schur", "updateleft", "updateright", "updateleft_schur",
    "updateright_schur", "updateleft_overlap", "updateright_overlap",
    "updateleft_scalar", "updateright_scalar",
    "l_LL_dense", "r_RR_dense", "l_LL_schur", "r_RR_schur",
    "simple_lanczos_solver", "stable_tsvd", "mps_truncate", "MPSTruncation",
    "leftorth_qr", "rightorth_lq", "krylov_exponentiate",
]

td = np.tensordot


# ---------------------------------------------------------------- H_eff * x
def ac_prime(x, W, L, R):
    """One-site H_eff*x, dense MPO.  algorithms/derivatives.jl:2-4

    tmp[-1 -2; -3] := ((hleft[-1,1,2] * x[2,3,4]) * m[1,-2,5,3]) * hright[-3,5,4]
    """
    t = td(L, x, axes=([2], [0]))            # [a', w, s, b]
    t = td(t, W, axes=([1, 2], [0, 3]))      # [a', b, s', w2]
    y = td(t, R, axes=([3, 1], [1, 2]))      # [a', s', b']
    return y


def ac2_prime(x, W1, W2, L, R):
    """Two-site H_eff*x, dense MPO.  algorithms/derivatives.jl:20-22

    tmp[-1 -2; -3 -4] := (((hleft[-1,1,2] * x[2,3,4,5]) * h1[1,-2,6,3])
                           * h2[6,-3,7,4]) * hright[-4,7,5]
    """
    t = td(L, x, axes=([2], [0]))            # [a', w, s1, s2, b]
    t = td(t, W1, axes=([1, 2], [0, 3]))     # [a', s2, b, s1', m]
    t = td(t, W2, axes=([4, 1], [0, 3]))     # [a', b, s1', s2', w2]
    y = td(t, R, axes=([4, 1], [1, 2]))      # [a', s1', s2', b']
    return y


def c_prime(C, L, R):
    """Zero-site H_eff*C.  algorithms/derivatives.jl:52-54

    tmp[-1; -2] := (hleft[-1,1,2] * x[2,3]) * hright[-2,1,3]
    """
    t = td(L, C, axes=([2], [0]))            # [a', w, b]
    return td(t, R, axes=([1, 2], [1, 2]))   # [a', b']


def _schur_blocks(W, tol=0.0):
    """Nonzero (i, j) blocks of a dense-embedded Schur MPO tensor, in the
    order of ``keys(h)`` (mpohamiltonian/abstractsitempo.jl:62, column-major
    Iterators.product order: i fastest)."""
    wl, _, wr, _ = W.shape
    out = []
    for j in range(wr):
        for i in range(wl):
            blk = W[i, :, j, :]
            if np.any(np.abs(blk) > tol):
                out.append((i, j, blk))
    return out


def ac_prime_schur(x, W, hleft, hright):
    """One-site H_eff*x, Schur form: sum over nonzero (i,j) blocks.
    algorithms/derivatives.jl:7-17 (scalar blocks handled as scal*identity,
    which the dense block already is)."""
    y = np.zeros_like(x, dtype=np.result_type(x, W, hleft, hright))
    for i, j, blk in _schur_blocks(W):
        # hleft[i][-1,5,4]*x[4,2,1]*ham[i,j][5,-2,3,2]*hright[j][-3,3,1]
        t = td(hleft[:, i, :], x, axes=([1], [0]))       # [a', s, b]
        t = td(t, blk, axes=([1], [1]))                  # [a', b, s']
        t = td(t, hright[:, j, :], axes=([1], [1]))      # [a', s', b']
        y += t
    return y


def ac2_prime_schur(x, W1, W2, hleft, hright):
    """Two-site H_eff*x, Schur form (algorithms/derivatives.jl:24-49): loops
    over (i,j) in keys(h1) and k with contains(h2,j,k); each chain is an
    independent contraction of hleft[i], x, h1[i,j], h2[j,k], hright[k]."""
    y = np.zeros(x.shape, dtype=np.result_type(x, W1, W2, hleft, hright))
    wr2 = W2.shape[2]
    for i, j, b1 in _schur_blocks(W1):
        for k in range(wr2):
            b2 = W2[j, :, k, :]
            if not np.any(b2 != 0):
                continue
            t = td(hleft[:, i, :], x, axes=([1], [0]))   # [a', s1, s2, b]
            t = td(t, b1, axes=([1], [1]))               # [a', s2, b, s1']
            t = td(t, b2, axes=([1], [1]))               # [a', b, s1', s2']
            t = td(t, hright[:, k, :], axes=([1], [1]))  # [a', s1', s2', b']
            y += t
    return y


def c_prime_schur(C, hleft, hright):
    """algorithms/derivatives.jl:56-63 (sum over w of L_w C R_w^T)."""
    y = np.zeros(C.shape, dtype=np.result_type(C, hleft, hright))
    for w in range(hleft.shape[1]):
        y += (hleft[:, w, :] @ C) @ hright[:, w, :].T
    return y


# ------------------------------------------------------ environment updates
def updateleft(hold, A, W, B):
    """mpo/transfer.jl:31-34

    hnew[-1; -2 -3] := hold[1,2,3] * psiBj[3,4,-3] * hj[2,5,-2,4] * conj(psiAj[1,5,-1])
    """
    t = td(hold, B, axes=([2], [0]))             # [a', w, s, b]
    t = td(t, W, axes=([1, 2], [0, 3]))          # [a', b, s', w2]
    t = td(t, np.conj(A), axes=([0, 2], [0, 1]))  # [b, w2, b']
    return np.transpose(t, (2, 1, 0))            # [b', w2, b]


def updateright(hold, A, W, B):
    """mpo/transfer.jl:26-29

    hnew[-1; -2 -3] := hold[1,2,3] * psiBj[-3,4,3] * hj[-2,5,2,4] * conj(psiAj[-1,5,1])
    """
    t = td(hold, B, axes=([2], [2]))             # [b', w2, a, s]
    t = td(t, W, axes=([1, 3], [2, 3]))          # [b', a, w, s']
    t = td(t, np.conj(A), axes=([0, 3], [2, 1]))  # [a, w, a']
    return np.transpose(t, (2, 1, 0))            # [a', w, a]


def updateleft_overlap(hold, A, B):
    """Operator-less update of a rank-3 environment, mpo/transfer.jl:42-45."""
    t = td(hold, B, axes=([2], [0]))             # [a', w, s, b]
    t = td(t, np.conj(A), axes=([0, 2], [0, 1]))  # [w, b, b']
    return np.transpose(t, (2, 0, 1))


def updateright_overlap(hold, A, B):
    """mpo/transfer.jl:37-40"""
    t = td(hold, B, axes=([2], [2]))             # [b', w, a, s]
    t = td(t, np.conj(A), axes=([0, 3], [2, 1]))  # [w, a, a']
    return np.transpose(t, (2, 0, 1))


def updateleft_scalar(hold, A, hj, B):
    """mpo/transfer.jl:52-55"""
    return hj * updateleft_overlap(hold, A, B)


def updateright_scalar(hold, A, hj, B):
    """mpo/transfer.jl:47-50"""
    return hj * updateright_overlap(hold, A, B)


def updateleft_schur(hold, A, W, B):
    """mpohamiltonian/transfer.jl:62-75: hnew[j] += update(hold[i], ..) over keys."""
    wr = W.shape[2]
    Dr = B.shape[2]
    T = np.result_type(hold, A, W, B)
    hnew = np.zeros((A.shape[2], wr, Dr), dtype=T)
    for i, j, blk in _schur_blocks(W):
        hnew[:, j, :] += updateleft(hold[:, i:i + 1, :], A, blk[None, :, None, :], B)[:, 0, :]
    return hnew


def updateright_schur(hold, A, W, B):
    """mpohamiltonian/transfer.jl:48-60"""
    wl = W.shape[0]
    T = np.result_type(hold, A, W, B)
    hnew = np.zeros((A.shape[0], wl, B.shape[0]), dtype=T)
    for i, j, blk in _schur_blocks(W):
        hnew[:, i, :] += updateright(hold[:, j:j + 1, :], A, blk[None, :, None, :], B)[:, 0, :]
    return hnew


def l_LL_dense(dtype=np.float64):
    """Left boundary of a strict FiniteMPO: a 1x1x1 isometry
    (mpo/arithmetics.jl:258-259, auxiliary/others.jl loose_isometry)."""
    return np.ones((1, 1, 1), dtype=dtype)


def r_RR_dense(dtype=np.float64):
    """mpo/arithmetics.jl:254-255"""
    return np.ones((1, 1, 1), dtype=dtype)


def l_LL_schur(w, dtype=np.float64):
    """Schur-form left boundary: ones at w=1, zeros elsewhere
    (mpohamiltonian/transfer.jl:26-44)."""
    e = np.zeros((1, w, 1), dtype=dtype)
    e[0, 0, 0] = 1
    return e


def r_RR_schur(w, dtype=np.float64):
    """Schur-form right boundary: ones at w=last (mpohamiltonian/transfer.jl:3-23)."""
    e = np.zeros((1, w, 1), dtype=dtype)
    e[0, w - 1, 0] = 1
    return e


# ------------------------------------------------------------------ Lanczos
LANCZOS_ORTH_TOL = 1.0e-12   # auxiliary/simple_lanczos.jl:1


def _dot(a, b):
    return np.vdot(a, b)       # Julia dot(a, b) conjugates the first argument


def simple_lanczos_solver(A, v, kmax=10, btol=1.0e-8, which="SR"):
    """auxiliary/simple_lanczos.jl:83-120 (with the first step :27-42 and the
    step :49-68).  Plain three-term recurrence, no reorthogonalisation; stops
    when beta < btol; lowest Ritz pair from eigen(Symmetric(T)).

    Returns (eigval, eigvec, info, k) where k is the Krylov dimension used.
    """
    if which not in ("SR", "SA"):
        raise ValueError("only the lowest eigenpair is restated")
    info = 0
    # lanczos_make_first_step
    vm = np.linalg.norm(v)
    qm1 = v / vm
    qi = A(qm1)
    a = _dot(qm1, qi)
    a = float(np.real(a))
    qi = qi - qm1 * a
    b = float(np.linalg.norm(qi))
    if b != 0.0:
        qi = qi / b
    if b < btol:
        return a, qm1, info, 1
    V = [qm1]
    T = np.zeros((kmax, kmax))
    T[0, 0] = a
    k = 1
    converged = False
    while k < kmax:
        T[k - 1, k] = b
        T[k, k - 1] = b
        # lanczos_make_step(A, qiminus1, qi, bold=b)
        qp1 = A(qi)
        a = float(np.real(_dot(qi, qp1)))
        qp1 = qp1 - (qi * a + qm1 * b)
        b = float(np.linalg.norm(qp1))
        if b != 0.0:
            qp1 = qp1 / b
        qm1 = qi
        qi = qp1
        V.append(qm1)
        T[k, k] = a
        k += 1
        if b < btol:
            converged = True
            break
    if not converged:
        info = -1
    w, U = scipy.linalg.eigh(T[:k, :k])
    y = U[:, 0]
    # lanczos_linear_transformation_single (:70-78): last term first
    evec = V[-1] * y[-1]
    for i in range(len(V) - 1):
        evec = evec + V[i] * y[i]
    return float(w[0]), evec, info, k


# ---------------------------------------------------------- truncated SVD
class MPSTruncation:
    """auxiliary/truncation.jl:8-16: drop sigma below eps*||sigma||_2 first,
    then keep at most D."""

    def __init__(self, D, eps, verbosity=0):
        self.D = int(D)
        self.eps = float(eps)
        self.verbosity = verbosity


def mps_truncate(s, trunc, p=2):
    """TensorKit._truncate!(v, ::MPSTruncation, p) -- auxiliary/truncation.jl:27-47.
    ``s`` is sorted descending.  Returns (kept count, err)."""
    n = np.linalg.norm(s, p)
    keep = int(np.count_nonzero(s >= trunc.eps * n))
    err1 = np.linalg.norm(s[keep:], p)
    if keep <= trunc.D:
        return keep, float(np.linalg.norm([err1], p))
    err2 = np.linalg.norm(s[trunc.D:keep], p)
    return trunc.D, float(np.linalg.norm([err1, err2], p))


def stable_tsvd(M, trunc=None):
    """auxiliary/stable_svd.jl:12-18: gesdd, falling back to gesvd."""
    try:
        u, s, vh = scipy.linalg.svd(M, full_matrices=False, lapack_driver="gesdd")
    except (np.linalg.LinAlgError, ValueError):
        u, s, vh = scipy.linalg.svd(M, full_matrices=False, lapack_driver="gesvd")
    if trunc is None:
        return u, s, vh, 0.0
    k, err = mps_truncate(s, trunc)
    return u[:, :k], s[:k], vh[:k, :], err


def leftorth_qr(A):
    """leftorth!(A, alg=QR()) on a site tensor A[a,s,b] viewed as (a s) x b.
    Returns Q[a,s,k], R[k,b] (algorithms/dmrg.jl:45, tdvp.jl:33)."""
    Dl, d, Dr = A.shape
    M = A.reshape(Dl * d, Dr, order="F")
    Q, R = np.linalg.qr(M, mode="reduced")
    return Q.reshape(Dl, d, Q.shape[1], order="F"), R


def rightorth_lq(A):
    """rightorth(A, (1,), (2,3), alg=LQ()) on A[a,s,b] viewed as a x (s b).
    Returns L[a,k], Q[k,s,b] (algorithms/dmrg.jl:69, tdvp.jl:55)."""
    Dl, d, Dr = A.shape
    M = A.reshape(Dl, d * Dr, order="F")
    Q, R = np.linalg.qr(M.T, mode="reduced")     # M^T = Q R  ->  M = R^T Q^T
    Lm = R.T
    Qm = Q.T
    return Lm, Qm.reshape(Qm.shape[0], d, Dr, order="F")


# ------------------------------------------------------- Krylov exponential
def krylov_exponentiate(A, t, v, tol=1e-12, krylovdim=30, maxiter=1000):
    """exp(t*A) v for Hermitian A by Krylov projection with adaptive time
    stepping (the published Expokit scheme, Sidje 1998).  This restates what
    KrylovKit.exponentiate computes (called at algorithms/tdvp.jl:4 with
    tol/abs(dt)); KrylovKit is an unpinned, un-vendored dependency, so the
    oracle only promises exp(t*A) v to ``tol`` per unit time."""
    v = np.asarray(v)
    beta = np.linalg.norm(v)
    if beta == 0:
        return np.zeros_like(v, dtype=np.result_type(v, t, 1j))
    w = v.astype(np.result_type(v, t, np.complex128)) / beta
    tau_total = abs(t)
    sgn = t / tau_total if tau_total != 0 else 1.0
    tau_done = 0.0
    dtau = tau_total
    out_scale = beta
    it = 0
    while tau_done < tau_total * (1 - 1e-15) and it < maxiter:
        it += 1
        V = [w]
        H = np.zeros((krylovdim + 1, krylovdim), dtype=np.complex128)
        m = krylovdim
        happy = False
        for j in range(krylovdim):
            z = A(V[j]).astype(np.complex128)
            for i in range(j + 1):                         # full orthogonalisation
                H[i, j] = np.vdot(V[i], z)
                z = z - H[i, j] * V[i]
            for i in range(j + 1):                         # second pass
                c = np.vdot(V[i], z)
                H[i, j] += c
                z = z - c * V[i]
            h = np.linalg.norm(z)
            H[j + 1, j] = h
            if h < 1e-14 * max(1.0, np.abs(H[:j + 1, :j + 1]).max()):
                m = j + 1
                happy = True
                break
            V.append(z / h)
        dtau = (tau_total - tau_done) if happy else min(dtau, tau_total - tau_done)
        while True:
            Hm = H[:m, :m] * (sgn * dtau)
            E = scipy.linalg.expm(Hm)
            if happy:
                err = 0.0
            else:
                # error estimate: |h_{m+1,m} * dtau * [exp(dtau H)]_{m,1}|
                err = abs(H[m, m - 1] * dtau * E[m - 1, 0])
            if err <= 0.9 * tol * dtau or dtau < 1e-300:
                break
            dtau *= 0.5
        c = E[:, 0]
        w = sum(c[i] * V[i] for i in range(m))
        nrm = np.linalg.norm(w)
        out_scale *= nrm
        w = w / nrm
        tau_done += dtau
        if not happy:
            dtau = min(2 * dtau, tau_total - tau_done) if tau_done < tau_total else dtau
    return w * out_scale
