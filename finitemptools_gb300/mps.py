"""FiniteMPS on the device (mps/finitemps.jl, mps/initializers.jl, mps/orth.jl).

Site numbering follows the reference: ``psi[1] .. psi[L]`` (1-based), bond
singular values ``psi.s[1] .. psi.s[L+1]``.
"""

import numpy as np

from .auxiliary import gemm, norm, scal, scale_cols, scale_rows, stable_tsvd
from .device import DeviceTensor, default_handle

__all__ = ["OneBased", "FiniteMPS", "randommps", "prodmps", "max_bond_dimensions",
           "canonicalize_", "increase_bond_", "bond_dimension"]


class OneBased:
    """A Python list indexed 1..n like the reference's Julia vectors."""

    def __init__(self, items):
        self._d = list(items)

    def __getitem__(self, i):
        if isinstance(i, slice):
            raise TypeError("OneBased does not slice")
        if i < 1 or i > len(self._d):
            raise IndexError("BoundsError: index %d of 1..%d" % (i, len(self._d)))
        return self._d[i - 1]

    def __setitem__(self, i, v):
        if i < 1 or i > len(self._d):
            raise IndexError("BoundsError: index %d of 1..%d" % (i, len(self._d)))
        self._d[i - 1] = v

    def __len__(self):
        return len(self._d)

    def __iter__(self):
        return iter(self._d)

    def tolist(self):
        return list(self._d)


class FiniteMPS:
    """struct FiniteMPS (mps/finitemps.jl:19-22): site tensors A[a, s, b] and
    bond singular values."""

    def __init__(self, data, svectors=None):
        self.data = OneBased(data)
        L = len(self.data)
        self.s = OneBased(svectors if svectors is not None else [None] * (L + 1))
        for i in range(1, L):
            if self.data[i].shape[2] != self.data[i + 1].shape[0]:
                raise ValueError("SpaceMismatch: bond %d" % i)

    def __len__(self):
        return len(self.data)

    def __getitem__(self, i):
        return self.data[i]

    def __setitem__(self, i, v):
        self.data[i] = v

    def __iter__(self):
        return iter(self.data)

    @property
    def dtype(self):
        return self.data[1].dtype

    @property
    def handle(self):
        return self.data[1].h

    def copy(self):
        return FiniteMPS([A.copy() for A in self.data],
                         [None if s is None else s.copy() for s in self.s])

    def to_numpy(self):
        return [A.numpy() for A in self.data]

    @staticmethod
    def from_numpy(tensors, handle=None, dtype=None):
        return FiniteMPS([DeviceTensor.from_numpy(A, handle, dtype) for A in tensors])


def max_bond_dimensions(ds, D):
    """max_bond_dimensions(physpaces::Vector{Int}, D) (finitemps.jl:283-297)."""
    L = len(ds)
    v = [1] * (L + 1)
    for i in range(1, L):
        v[i] = min(v[i - 1] * ds[i - 1], D)
    v[L] = 1
    for i in range(L - 1, 0, -1):
        v[i] = min(v[i], ds[i] * v[i + 1])
    return v


def randommps(L, d, D, rng=None, dtype=np.float64, handle=None):
    """randommps(T, L; d, D) (mps/initializers.jl:101-108): iid N(0,1) site
    tensors on the maximal virtual spaces capped at D.  ``rng`` is a numpy
    Generator; entries are drawn per site in column-major order (complex:
    real plane then imaginary plane, each scaled by 1/sqrt(2))."""
    rng = rng if rng is not None else np.random.default_rng()
    v = max_bond_dimensions([d] * L, D)
    out = []
    for i in range(L):
        shape = (v[i], d, v[i + 1])
        n = int(np.prod(shape))
        if np.issubdtype(np.dtype(dtype), np.complexfloating):
            flat = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2.0)
        else:
            flat = rng.standard_normal(n)
        out.append(DeviceTensor.from_numpy(flat.reshape(shape, order="F"), handle, dtype))
    return FiniteMPS(out)


def prodmps(vectors, dtype=np.float64, handle=None):
    """prodmps(physectors::Vector{Vector}) (mps/initializers.jl:80-87)."""
    return FiniteMPS([DeviceTensor.from_numpy(np.asarray(v, dtype=dtype).reshape(1, len(v), 1),
                                              handle, dtype) for v in vectors])


def bond_dimension(psi):
    return max(psi[i].shape[2] for i in range(1, len(psi)))


def canonicalize_(psi, normalize=False):
    """right_canonicalize! (mps/orth.jl:40-49): SVD leftorth! sweep, optional
    normalisation of the last site, SVD rightorth! sweep (no truncation)."""
    L = len(psi)
    # maybe_init_boundary_s! (finitemps.jl:179-189): identities on the open ends
    if psi.s[1] is None:
        psi.s[1] = DeviceTensor.from_numpy(np.ones(psi[1].shape[0]), psi.handle, np.float64)
    if psi.s[L + 1] is None:
        psi.s[L + 1] = DeviceTensor.from_numpy(np.ones(psi[L].shape[2]), psi.handle, np.float64)
    for i in range(1, L):                                    # orth.jl:5-20
        A = psi[i]
        Dl, d, Dr = A.shape
        u, s, vt, _ = stable_tsvd(A, Dl * d, Dr)
        k = s.shape[0]
        psi[i] = u.view_as((Dl, d, k))
        scale_rows(vt, k, Dr, s)                             # v2 = s * v
        B = psi[i + 1]
        psi[i + 1] = gemm(vt, B, (k, B.shape[1], B.shape[2]), k, B.shape[1] * B.shape[2], Dr)
        psi.s[i + 1] = s
    if normalize:
        nrm = norm(psi[L])
        scal(1.0 / nrm, psi[L])
    for i in range(L, 1, -1):                                # orth.jl:22-37
        A = psi[i]
        Dl, d, Dr = A.shape
        u, s, vt, _ = stable_tsvd(A, Dl, d * Dr)
        k = s.shape[0]
        psi[i] = vt.view_as((k, d, Dr))
        scale_cols(u, Dl, k, s)                              # u2 = u * s
        P = psi[i - 1]
        psi[i - 1] = gemm(P, u, (P.shape[0], P.shape[1], k), P.shape[0] * P.shape[1], k, Dl)
        psi.s[i] = s
    return psi


def increase_bond_(psi, D):
    """increase_bond!(psi::FiniteNonSymmetricMPS; D) (finitemps.jl:302-317):
    zero-pad the site tensors to the capped maximal virtual dimensions."""
    if bond_dimension(psi) >= D:
        return psi
    ds = [psi[i].shape[1] for i in range(1, len(psi) + 1)]
    v = max_bond_dimensions(ds, D)
    for i in range(1, len(psi) + 1):
        A = psi[i].numpy()
        sl = max(min(v[i - 1], D), A.shape[0])
        sr = max(min(v[i], D), A.shape[2])
        m = np.zeros((sl, A.shape[1], sr), dtype=A.dtype)
        m[:A.shape[0], :, :A.shape[2]] = A
        psi[i] = DeviceTensor.from_numpy(m, psi[i].h, psi[i].dtype)
    return psi
