"""Restatement of exact diagonalisation and exact time evolution on
ExactFiniteMPS (test infrastructure only: the product never imports this
module).

- max_bond_dimensions: mps/finitemps.jl:257-273 (no symmetry);
- _find_center, _exactmps_side_tensors, ExactFiniteMPS(randn, ...),
  ExactFiniteMPS(psi): mps/exactmps.jl:79-141;
- init_h_center, exact_diagonalization, exact_timeevolution:
  algorithms/exactdiag.jl:3-61.
KrylovKit's eigsolve / exponentiate are not vendored; they are restated by
ARPACK's implicitly restarted Lanczos (scipy.sparse.linalg.eigsh) and the
Al-Mohy & Higham truncated Taylor action (scipy.sparse.linalg.expm_multiply)
on the same linear map.  Site numbers are 1-based, lists 0-based.
"""

import numpy as np
import scipy.sparse.linalg as spla

from .core import ac_prime, l_LL_dense, l_LL_schur, r_RR_dense, r_RR_schur, updateleft, updateright
from .excited import c_proj, overlap_updateleft, overlap_updateright

__all__ = ["max_bond_dimensions", "find_center", "side_tensors", "random_exact_mps",
           "exact_mps_from", "init_h_center", "exact_diagonalization", "exact_timeevolution"]


def max_bond_dimensions(physdims):
    L = len(physdims)
    Ds = [1] * (L + 1)
    left = 1
    for i in range(1, L + 1):                  # Julia for i in 1:L
        left *= physdims[i - 1]
        Ds[i] = left                           # Ds[i+1] (1-based)
    Ds[L] = 1
    right = 1
    for i in range(L, 0, -1):                  # Julia for i in L:-1:1
        right *= physdims[i - 1]
        Ds[i - 1] = min(Ds[i - 1], right)
    return Ds


def find_center(Ds):
    """1-based bond positions as in Julia: pos = argmax(Ds); step left when
    Ds[pos-1] >= Ds[pos+1]."""
    pos = int(np.argmax(Ds)) + 1
    if pos != 1 and Ds[pos - 2] >= Ds[pos]:
        pos -= 1
    return pos


def side_tensors(physdims, dtype=np.float64):
    L = len(physdims)
    mid = find_center(max_bond_dimensions(physdims))
    out = [None] * L
    left = 1
    for i in range(1, mid):
        d = physdims[i - 1]
        # isomorphism(left (x) phys, fuse(left, phys)): column-major fusion a + left*s
        out[i - 1] = np.eye(left * d, dtype=dtype).reshape(left, d, left * d, order="F")
        left *= d
    right = 1
    for i in range(L, mid, -1):
        d = physdims[i - 1]
        # permute(isomorphism(fuse(phys', right), phys' (x) right), (1, 2), (3,))
        out[i - 1] = np.eye(d * right, dtype=dtype).reshape(d * right, d, right, order="F")
        right *= d
    return out, left, right, mid


def random_exact_mps(physdims, rng, dtype=np.float64):
    out, left, right, mid = side_tensors(physdims, dtype)
    C = rng.standard_normal((left, physdims[mid - 1], right))
    if dtype == np.complex128:
        C = C + 1j * rng.standard_normal(C.shape)
    out[mid - 1] = C.astype(dtype)
    return out, mid


def exact_mps_from(psi):
    """ExactFiniteMPS(psi::FiniteMPS) (exactmps.jl:124-141)."""
    L = len(psi)
    physdims = [A.shape[1] for A in psi]
    T = np.result_type(*psi)
    out, _, _, mid = side_tensors(physdims, T)
    cleft = np.eye(psi[0].shape[0], dtype=T)
    cright = np.eye(psi[-1].shape[2], dtype=T)
    for i in range(1, mid):
        cleft = overlap_updateleft(cleft, out[i - 1], psi[i - 1])
    for i in range(L, mid, -1):
        cright = overlap_updateright(cright, out[i - 1], psi[i - 1])
    out[mid - 1] = c_proj(psi[mid - 1], cleft, cright)
    return out, mid


def init_h_center(Ws, mps, mid, schur=False):
    """init_h_center (exactdiag.jl:3-18)."""
    L = len(mps)
    T = np.result_type(mps[mid - 1], *Ws)
    if schur:
        left, right = l_LL_schur(Ws[0].shape[0], T), r_RR_schur(Ws[-1].shape[2], T)
    else:
        left, right = l_LL_dense(T), r_RR_dense(T)
    for i in range(L, mid, -1):
        right = updateright(right, mps[i - 1], Ws[i - 1], mps[i - 1])
    for i in range(1, mid):
        left = updateleft(left, mps[i - 1], Ws[i - 1], mps[i - 1])
    return left, right


def _linear_map(Ws, mps, mid, schur):
    left, right = init_h_center(Ws, mps, mid, schur)
    shape = mps[mid - 1].shape
    W = Ws[mid - 1]
    T = np.result_type(mps[mid - 1], W, left, right)
    n = int(np.prod(shape))

    def mv(v):
        return ac_prime(np.asarray(v).reshape(shape, order="F"), W, left, right).ravel(order="F")

    # Hermitian: the adjoint action (for the norm estimates of expm_multiply) is mv
    return spla.LinearOperator((n, n), matvec=mv, rmatvec=mv, dtype=T), shape


def exact_diagonalization(Ws, num=1, rng=None, schur=False, tol=1e-12):
    """exact_diagonalization(h; num, ishermitian=true) (exactdiag.jl:23-42)."""
    rng = rng or np.random.default_rng(0)
    physdims = [W.shape[1] for W in Ws]
    T = np.result_type(*Ws)
    mps, mid = random_exact_mps(physdims, rng, np.complex128 if T == np.complex128 else np.float64)
    A, shape = _linear_map(Ws, mps, mid, schur)
    vals, vecs = spla.eigsh(A, k=num, which="SA", v0=mps[mid - 1].ravel(order="F"), tol=tol)
    order = np.argsort(vals)
    states = []
    for i in order:
        st = list(mps)
        st[mid - 1] = vecs[:, i].reshape(shape, order="F")
        states.append(st)
    return vals[order], states, mid


def exact_timeevolution(Ws, t, mps, mid, schur=False):
    """exact_timeevolution(h, t, psi; ishermitian=true) (exactdiag.jl:44-61)."""
    mps = [np.asarray(A, dtype=np.complex128) for A in mps]
    A, shape = _linear_map(Ws, mps, mid, schur)
    At = spla.LinearOperator(A.shape, matvec=lambda v: t * A.matvec(v),
                             rmatvec=lambda v: np.conj(t) * A.matvec(v), dtype=np.complex128)
    y = spla.expm_multiply(At, mps[mid - 1].ravel(order="F"), traceA=0.0)
    out = list(mps)
    out[mid - 1] = y.reshape(shape, order="F")
    return out
