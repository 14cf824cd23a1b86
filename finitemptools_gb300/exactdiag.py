"""Exact diagonalisation and exact time evolution through the device one-site
H_eff (algorithms/exactdiag.jl:3-61) on ExactFiniteMPS (mps/exactmps.jl).

An ExactFiniteMPS keeps the whole state in its centre tensor.  Left of the
centre every site tensor is the identity map left (x) phys -> fused, right of
it the identity map fused -> phys (x) right, so the environments at the centre
are the complete left and right blocks of the Hamiltonian, and ac_prime at the
centre is H itself, applied as dense GEMMs on the device.  The centre is the
site next to the largest bond (_find_center, exactmps.jl:79-85).  Spaces carry
no symmetry here, so the sector argument of the reference is the trivial one.
"""

import numpy as np

from .derivatives import HeffOp
from .device import DeviceTensor
from .envs import _mpo_tensors, l_LL, r_RR
from .excited import c_proj, overlap_updateleft, overlap_updateright
from .mps import FiniteMPS, OneBased
from .transfer import updateleft, updateright
from .utilities import MPOHamiltonian

__all__ = ["ExactFiniteMPS", "max_bond_dimensions", "find_center", "init_h_center",
           "exact_diagonalization", "exact_timeevolution"]


def max_bond_dimensions(physdims):
    """max_bond_dimensions(physpaces, sector) without symmetry
    (mps/finitemps.jl:257-273): 0-based list of the L+1 bond dimensions."""
    L = len(physdims)
    Ds = [1] * (L + 1)
    left = 1
    for i in range(L):
        left *= int(physdims[i])
        Ds[i + 1] = left
    Ds[L] = 1
    right = 1
    for i in range(L - 1, -1, -1):
        right *= int(physdims[i])
        Ds[i] = min(Ds[i], right)
    return Ds


def find_center(Ds):
    """_find_center (exactmps.jl:79-85) on the 0-based bond list; returns the
    1-based centre site."""
    pos = int(np.argmax(Ds))                   # first maximum, 0-based bond = site pos+1's left bond
    if pos != 0 and Ds[pos - 1] >= Ds[pos + 1]:
        pos -= 1
    return pos + 1


def _side_tensors(physdims, dtype, handle):
    """_exactmps_side_tensors (exactmps.jl:87-106): identity maps
    A[a, s, a + Dl*s] left of the centre and B[s + d*b, s, b] right of it."""
    L = len(physdims)
    mid = find_center(max_bond_dimensions(physdims))
    tensors = [None] * L
    left = 1
    for i in range(mid - 1):
        d = int(physdims[i])
        A = np.zeros((left, d, left * d), dtype=dtype)
        a, s = np.meshgrid(np.arange(left), np.arange(d), indexing="ij")
        A[a, s, a + left * s] = 1
        tensors[i] = DeviceTensor.from_numpy(A, handle, dtype)
        left *= d
    right = 1
    for i in range(L - 1, mid - 1, -1):
        d = int(physdims[i])
        B = np.zeros((d * right, d, right), dtype=dtype)
        s, b = np.meshgrid(np.arange(d), np.arange(right), indexing="ij")
        B[s + d * b, s, b] = 1
        tensors[i] = DeviceTensor.from_numpy(B, handle, dtype)
        right *= d
    return tensors, left, right, mid


class ExactFiniteMPS:
    """struct ExactFiniteMPS (exactmps.jl:1-10): ``data`` 1-based, only the centre
    tensor may be replaced (setindex!, :27-33)."""

    def __init__(self, data, center):
        self.data = OneBased(list(data))
        self.center = int(center)

    @staticmethod
    def random(physdims, dtype=np.float64, rng=None, handle=None):
        """ExactFiniteMPS(randn, T, physpaces) (exactmps.jl:117-122)."""
        rng = rng or np.random.default_rng()
        tensors, left, right, mid = _side_tensors(physdims, dtype, handle)
        C = rng.standard_normal((left, int(physdims[mid - 1]), right))
        if np.dtype(dtype) == np.complex128:
            C = C + 1j * rng.standard_normal(C.shape)
        tensors[mid - 1] = DeviceTensor.from_numpy(C, handle, dtype)
        return ExactFiniteMPS(tensors, mid)

    @staticmethod
    def from_mps(psi):
        """ExactFiniteMPS(psi::FiniteMPS) (exactmps.jl:124-141): the centre is the
        projection of psi onto the exact basis (overlap chains and c_proj)."""
        L = len(psi)
        if psi[1].shape[0] != 1 or psi[L].shape[2] != 1:
            raise ValueError("only strict mps allowed")
        physdims = [psi[i].shape[1] for i in range(1, L + 1)]
        tensors, _, _, mid = _side_tensors(physdims, psi.dtype, psi.handle)
        one = DeviceTensor.from_numpy(np.ones((1, 1)), psi.handle, psi.dtype)
        cleft, cright = one, one.copy()
        for i in range(1, mid):
            cleft = overlap_updateleft(cleft, tensors[i - 1], psi[i])
        for i in range(L, mid, -1):
            cright = overlap_updateright(cright, tensors[i - 1], psi[i])
        tensors[mid - 1] = c_proj(psi[mid], cleft, cright)
        return ExactFiniteMPS(tensors, mid)

    def __len__(self):
        return len(self.data)

    def __getitem__(self, i):
        return self.data[i]

    def __setitem__(self, i, v):
        if i != self.center:
            raise ValueError("only center can be set.")
        if tuple(v.shape) != tuple(self.data[i].shape):
            raise ValueError("SpaceMismatch")
        self.data[i] = v

    @property
    def dtype(self):
        return self.data[self.center].dtype

    @property
    def handle(self):
        return self.data[self.center].h

    def copy(self):
        """copy(psi) (exactmps.jl:35): the side tensors are shared, as in the
        reference's shallow copy of the data vector."""
        return ExactFiniteMPS([self.data[i] for i in range(1, len(self) + 1)], self.center)

    def to_finite_mps(self):
        """FiniteMPS(psi::ExactFiniteMPS) (exactmps.jl:77)."""
        return FiniteMPS([self.data[i] for i in range(1, len(self) + 1)])

    def astype(self, dtype):
        if np.dtype(dtype) == self.dtype:
            return self
        return ExactFiniteMPS([DeviceTensor.from_numpy(self.data[i].numpy(), self.handle, dtype)
                               for i in range(1, len(self) + 1)], self.center)


def _sites(h, L):
    Ws, schur = _mpo_tensors(h, L)
    return [np.asarray(W) for W in Ws], schur


def _default_len(h):
    """_default_len (exactdiag.jl:20-21): length(h) of a FiniteMPO, the period of
    an MPOHamiltonian."""
    return h.period() if isinstance(h, MPOHamiltonian) else len(h)


def init_h_center(h, psi, precision="fp64"):
    """init_h_center (exactdiag.jl:3-18): the full left and right environments
    of the centre site."""
    L = len(psi)
    Ws, schur = _sites(h, L)
    cplx = psi.dtype == np.complex128 or any(np.iscomplexobj(W) for W in Ws)
    dt = np.complex128 if cplx else np.float64
    if psi.dtype != dt:
        raise TypeError("a complex MPO needs a complex ExactFiniteMPS")
    Ws = [W.astype(dt) for W in Ws]
    hd = psi.handle
    mid = psi.center
    right = r_RR(Ws[-1].shape[2], dt, hd, schur)
    for i in range(L, mid, -1):
        right = updateright(right, psi[i], Ws[i - 1], psi[i], precision)
    left = l_LL(Ws[0].shape[0], dt, hd, schur)
    for i in range(1, mid):
        left = updateleft(left, psi[i], Ws[i - 1], psi[i], precision)
    return left, right, Ws[mid - 1]


_ORDER = {"SR": lambda v: v.real, "LR": lambda v: -v.real, "LM": lambda v: -np.abs(v),
          "SM": lambda v: np.abs(v), "SI": lambda v: v.imag, "LI": lambda v: -v.imag}


def _arnoldi_eigsolve(op, x0, num, which, krylovdim, maxiter, tol):
    """eigsolve(f, x0, num, which, Arnoldi()) for a non-Hermitian f (exactdiag.jl:25-28):
    explicitly restarted Arnoldi on the device vectors (two-pass Gram-Schmidt through
    device dots and axpys).  The krylovdim x krylovdim Hessenberg eigenproblem is solved on
    the host, as KrylovKit solves its small dense problem; the restart vector is the sum of
    the wanted Ritz vectors.  Returns (values, vectors, info) like HeffOp.eigsolve."""
    from .auxiliary import axpy, dot, norm, scal
    if which not in _ORDER:
        raise ValueError("which must be one of %s" % sorted(_ORDER))
    m = max(num + 1, int(krylovdim))
    x = scal(1.0 / norm(x0), x0.copy())
    applies = 0
    for it in range(int(maxiter)):
        V = [x]
        H = np.zeros((m + 1, m), dtype=np.complex128)
        k = m
        for j in range(m):
            w = op(V[j])
            applies += 1
            for _ in range(2):
                for i in range(j + 1):
                    c = dot(V[i], w)
                    H[i, j] += c
                    axpy(-c, V[i], w)
            b = norm(w)
            H[j + 1, j] = b
            if b <= 1e-14 * max(1.0, np.abs(H[:j + 2, :j + 1]).max()):
                k = j + 1                              # invariant subspace
                break
            V.append(scal(1.0 / b, w))
        ev, Y = np.linalg.eig(H[:k, :k])
        idx = np.argsort(_ORDER[which](ev), kind="stable")[:num]
        res = np.abs(H[k, k - 1]) * np.abs(Y[k - 1, idx]) if k < len(V) else np.zeros(len(idx))
        vecs = []
        for i in idx:
            u = scal(complex(Y[0, i]), V[0].copy())
            for q in range(1, k):
                axpy(complex(Y[q, i]), V[q], u)
            vecs.append(scal(1.0 / norm(u), u))
        done = np.all(res <= tol * np.maximum(1.0, np.abs(ev[idx]))) or k < m
        if done or it == int(maxiter) - 1:
            info = {"converged": int(np.sum(res <= tol * np.maximum(1.0, np.abs(ev[idx])))),
                    "residuals": [float(r) for r in res], "applies": applies}
            return [complex(v) for v in ev[idx]], vecs, info
        x = vecs[0].copy()
        for u in vecs[1:]:
            axpy(1.0, u, x)
        x = scal(1.0 / norm(x), x)


def exact_diagonalization(h, len=None, ishermitian=True, num=1, which="SR", dtype=None,
                          rng=None, handle=None, krylovdim=30, maxiter=100, tol=1e-12,
                          precision="fp64"):
    """exact_diagonalization(h; sector, len, ishermitian, num, which)
    (exactdiag.jl:23-42): eigsolve of ac_prime at the centre of a random
    ExactFiniteMPS, by thick-restart Lanczos for Hermitian h and by restarted Arnoldi
    (complex vectors, complex eigenvalues) otherwise.  Returns (values, states)."""
    n_sites = len if len is not None else _default_len(h)
    Ws, _ = _sites(h, n_sites)
    physdims = [W.shape[1] for W in Ws]
    cplx = any(np.iscomplexobj(W) for W in Ws) or not ishermitian
    dt = np.dtype(dtype) if dtype is not None else np.dtype(np.complex128 if cplx else np.float64)
    if not ishermitian and dt != np.complex128:
        raise TypeError("non-Hermitian exact diagonalisation needs complex128 states")
    psi = ExactFiniteMPS.random(physdims, dt, rng, handle)
    left, right, Wc = init_h_center(h, psi, precision)
    op = HeffOp("ac", left, right, W1=Wc, precision=precision, dtype=dt)
    if ishermitian:
        vals, vecs, info = op.eigsolve(psi[psi.center], num, which, krylovdim, maxiter, tol)
    else:
        vals, vecs, info = _arnoldi_eigsolve(op, psi[psi.center], num, which, krylovdim,
                                             maxiter, tol)
    if info["converged"] < num:
        import warnings
        warnings.warn("only %d converged." % info["converged"])
    states = []
    for v in vecs:
        st = psi.copy()
        st[st.center] = v
        states.append(st)
    return vals, states


def exact_timeevolution(h, t, psi, ishermitian=True, tol=1e-12, krylovdim=30,
                        precision="fp64"):
    """exact_timeevolution(h, t, psi; ishermitian) (exactdiag.jl:44-61):
    exponentiate of ac_prime at the centre.  A complex t promotes the state to
    complex128.  Both values of ishermitian take the same solver: fmpt_exponentiate is an
    Arnoldi exponential (full two-pass Gram-Schmidt, exponential of the Hessenberg
    matrix), the reference's Arnoldi() driver, which its Lanczos() driver for Hermitian h
    matches up to rounding."""
    t = complex(t)
    if t.imag != 0.0:
        psi = psi.astype(np.complex128)
    left, right, Wc = init_h_center(h, psi, precision)
    op = HeffOp("ac", left, right, W1=Wc, precision=precision, dtype=psi.dtype)
    tt = t if psi.dtype == np.complex128 else t.real
    y = op.exponentiate(tt, psi[psi.center], tol / max(abs(t), 1e-300), krylovdim)
    out = psi.copy()
    out[out.center] = y
    return out
