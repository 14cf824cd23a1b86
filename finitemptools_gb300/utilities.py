"""Host-side operator data for the DMRG/TDVP path: site operators, Schur-form
MPO tensors, MPOHamiltonian and its dense FiniteMPO embedding.

These are one-off host constructions (no device work); the device path only
sees the dense W[wl, s_out, wr, s_in] tensors they produce plus the nonzero
(w, w') block pattern.  Conventions follow the reference:
  * spin-1/2 matrices          utilities/spin_siteops.jl:1-8
  * XXZ chain terms            utilities/models.jl:27-42
  * SchurMPOTensor grid        mpohamiltonian/schurmpotensor.jl:1-111
  * FiniteMPO(h, L) embedding  mpohamiltonian/mpohamiltonian.jl:101-130
"""

import numpy as np

__all__ = [
    "spin_half_matrices", "SchurMPOTensor", "MPOHamiltonian", "FiniteMPO",
    "heisenberg_xxz_mpo", "j1j2_heisenberg_mpo", "tfi_mpo",
]


def spin_half_matrices():
    """utilities/spin_siteops.jl:1-8 (Pauli matrices, s_Z = diag(-1, 1))."""
    sp = np.array([[0.0, 0.0], [1.0, 0.0]])
    sm = np.array([[0.0, 1.0], [0.0, 0.0]])
    z = np.array([[-1.0, 0.0], [0.0, 1.0]])
    x = sp + sm
    y = -1j * (sp - sm)
    return {"x": x, "y": y, "z": z, "+": sp, "-": sm}


class SchurMPOTensor:
    """Upper-triangular w x w grid of site operators or scalars
    (mpohamiltonian/schurmpotensor.jl:1-10).  ``Os[i][j]`` is a d x d matrix,
    a scalar (scalar times identity) or 0 (structurally absent)."""

    def __init__(self, Os):
        w = len(Os)
        if any(len(r) != w for r in Os):
            raise ValueError("Schur MPO grid must be square")
        d = None
        for i in range(w):
            for j in range(w):
                o = Os[i][j]
                if isinstance(o, np.ndarray):
                    if d is None:
                        d = o.shape[0]
                    elif o.shape != (d, d):
                        raise ValueError("physical dimension mismatch")
                    if i > j and np.any(o != 0):
                        raise ValueError("Canonical MPO Tensor is upper triangular.")
                elif i > j and o != 0:
                    raise ValueError("Canonical MPO Tensor is upper triangular.")
        if d is None:
            raise ValueError("there must be at least one operator in the grid")
        self.Os = Os
        self.w = w
        self.d = d

    def contains(self, i, j):
        """contains(m, i, j) (schurmpotensor.jl:110)."""
        o = self.Os[i][j]
        return i <= j and (np.any(o != 0) if isinstance(o, np.ndarray) else o != 0)

    def isscal(self, i, j):
        """isscal(m, i, j) (schurmpotensor.jl:111)."""
        return (not isinstance(self.Os[i][j], np.ndarray)) and self.contains(i, j)

    def keys(self):
        """keys(h) in Iterators.product order (i fastest), abstractsitempo.jl:62."""
        return [(i, j) for j in range(self.w) for i in range(self.w) if self.contains(i, j)]

    def dense(self, dtype=None):
        """Dense W[w, s_out, w', s_in] with the exact zero pattern."""
        dt = dtype or np.result_type(*[np.asarray(o) for r in self.Os for o in r], np.float64)
        W = np.zeros((self.w, self.d, self.w, self.d), dtype=dt)
        for i, j in self.keys():
            o = self.Os[i][j]
            W[i, :, j, :] = o if isinstance(o, np.ndarray) else o * np.eye(self.d)
        return W


class MPOHamiltonian:
    """Periodic chain of Schur tensors (mpohamiltonian/mpohamiltonian.jl:1-27)."""

    def __init__(self, data):
        if isinstance(data, SchurMPOTensor):
            data = [data]
        if not data:
            raise ValueError("empty data.")
        d = data[0].d
        for t in data:
            if t.d != d:
                raise ValueError("odim mismatch.")
        self.data = list(data)

    def period(self):
        return len(self.data)

    def __getitem__(self, i):
        """1-based periodic indexing as PeriodicArray."""
        return self.data[(i - 1) % len(self.data)]

    def site_tensors(self, L):
        """Dense bulk grids for sites 1..L (Schur environments keep the
        boundary vectors l_LL/r_RR instead of cutting the grid)."""
        if L % self.period():
            raise ValueError("length must be a multiple of the period")
        return [self[i].dense() for i in range(1, L + 1)]


def FiniteMPO(h, L):
    """FiniteMPO(h::MPOHamiltonian, L) (mpohamiltonian.jl:101-130): row 1 of
    the first grid, the full bulk grids, the last column of the last grid."""
    if L % h.period():
        raise ValueError("DimensionMismatch")
    if L < 2:
        raise ValueError("size of FiniteMPO must at least be 2.")
    Ws = h.site_tensors(L)
    Ws[0] = Ws[0][0:1]
    Ws[-1] = Ws[-1][:, :, -1:, :]
    return [np.ascontiguousarray(W) for W in Ws]


def heisenberg_xxz_mpo(J=1.0, Jzz=1.0, hz=0.0):
    """Schur MPO (w=5) of heisenberg_xxz_util's terms (models.jl:27-42):
    hz Z_i + 2J (S+_i S-_{i+1} + S-_i S+_{i+1}) + Jzz Z_i Z_{i+1}.
    Nonzero blocks (1,1),(1,2),(1,3),(1,4),(2,5),(3,5),(4,5),(5,5) [+(1,5) if hz]."""
    p = spin_half_matrices()
    sp, sm, z = p["+"], p["-"], p["z"]
    I = np.eye(2)
    O = [[0] * 5 for _ in range(5)]
    O[0][0] = I
    O[0][1] = 2 * J * sp
    O[0][2] = 2 * J * sm
    O[0][3] = Jzz * z
    O[0][4] = hz * z if hz != 0 else 0
    O[1][4] = sm
    O[2][4] = sp
    O[3][4] = z
    O[4][4] = I
    return MPOHamiltonian(SchurMPOTensor(O))


def j1j2_heisenberg_mpo(J1=1.0, J2=0.5):
    """Schur MPO (w=8) of J1 sum s_i.s_{i+1} + J2 sum s_i.s_{i+2} in the Pauli
    convention of models.jl (2J(S+S- + h.c.) + J ZZ per bond): identity,
    three one-site-pending, three two-site-pending channels, final."""
    p = spin_half_matrices()
    sp, sm, z = p["+"], p["-"], p["z"]
    I = np.eye(2)
    O = [[0] * 8 for _ in range(8)]
    O[0][0] = I
    O[0][1], O[0][2], O[0][3] = sp, sm, z
    O[1][4], O[2][5], O[3][6] = 1.0, 1.0, 1.0           # scalar*identity pass-through
    O[1][7], O[2][7], O[3][7] = 2 * J1 * sm, 2 * J1 * sp, J1 * z
    O[4][7], O[5][7], O[6][7] = 2 * J2 * sm, 2 * J2 * sp, J2 * z
    O[7][7] = I
    return MPOHamiltonian(SchurMPOTensor(O))


def tfi_mpo(h):
    """Schur MPO (w=3) of -sum Z_i Z_{i+1} - sum h_i X_i with site-dependent
    fields: an MPOHamiltonian whose period is the chain length."""
    p = spin_half_matrices()
    x, z = p["x"], p["z"]
    I = np.eye(2)
    data = []
    for hi in h:
        O = [[0] * 3 for _ in range(3)]
        O[0][0] = I
        O[0][1] = -z
        O[0][2] = -float(hi) * x
        O[1][2] = z
        O[2][2] = I
        data.append(SchurMPOTensor(O))
    return MPOHamiltonian(data)
