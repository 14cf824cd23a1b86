"""Exact references for the oracle pins (test infrastructure only).

The reference's tests pin DMRG energies to ``exact_diagonalization`` and TDVP
observables to ``exact_timeevolution`` (test/runtests.jl:773-790).  Those are
restated here independently of any MPO: Hamiltonians are built from their
terms by Kronecker products (site 1 is the fastest index, as in a
column-major reshape of the MPS chain), and the free-fermion closed form
covers the XX chain.
"""

import numpy as np
import scipy.linalg
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# utilities/spin_siteops.jl:1-8 (Pauli matrices, s_Z = diag(-1, 1))
SP = np.array([[0.0, 0.0], [1.0, 0.0]])
SM = np.array([[0.0, 1.0], [0.0, 0.0]])
SZ = np.array([[-1.0, 0.0], [0.0, 1.0]])
SX = SP + SM
I2 = np.eye(2)


def kron_chain(ops):
    """ops[0] acts on site 1 (fastest index)."""
    out = np.array([[1.0]])
    for o in ops:
        out = np.kron(o, out)
    return out


def dense_from_terms(L, d, terms):
    """terms: list of (coeff, {site(1-based): local matrix})."""
    n = d ** L
    H = np.zeros((n, n), dtype=np.result_type(*[np.asarray(c) for c, _ in terms], np.float64))
    for c, ops in terms:
        H += c * kron_chain([ops.get(i, np.eye(d)) for i in range(1, L + 1)])
    return H


# ----------------------------------------------------------- spin chains
def xxz_terms(L, J=1.0, Jzz=1.0, hz=0.0):
    """heisenberg_xxz_util (utilities/models.jl:27-42)."""
    terms = [(hz, {i: SZ}) for i in range(1, L + 1) if hz != 0]
    for i in range(1, L):
        terms.append((2 * J, {i: SP, i + 1: SM}))
        terms.append((2 * J, {i: SM, i + 1: SP}))
        terms.append((Jzz, {i: SZ, i + 1: SZ}))
    return terms


def _sz_sector_hamiltonian(L, bonds, hz=0.0, nup=None):
    """Sparse XXZ-type Hamiltonian in a fixed-magnetisation sector.
    bonds: list of (i, j, Jxy, Jzz) with 0-based sites; the flip amplitude of
    2*Jxy*(s+s- + h.c.) is 2*Jxy.  Bit k set = site k+1 in basis state 1
    (z = +1)."""
    nup = L // 2 if nup is None else nup
    states = np.array([s for s in range(1 << L) if bin(s).count("1") == nup], dtype=np.int64)
    index = {int(s): k for k, s in enumerate(states)}
    n = len(states)
    bits = ((states[:, None] >> np.arange(L)[None, :]) & 1).astype(np.int8)
    z = 2.0 * bits - 1.0
    diag = hz * z.sum(axis=1)
    rows, cols, vals = [], [], []
    for (i, j, jxy, jzz) in bonds:
        diag = diag + jzz * z[:, i] * z[:, j]
        anti = bits[:, i] != bits[:, j]
        src = np.nonzero(anti)[0]
        flipped = states[src] ^ ((1 << i) | (1 << j))
        dst = np.array([index[int(f)] for f in flipped], dtype=np.int64)
        rows.append(dst)
        cols.append(src)
        vals.append(np.full(len(src), 2.0 * jxy))
    rows.append(np.arange(n))
    cols.append(np.arange(n))
    vals.append(diag)
    H = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    return H


def xxz_ground_energy(L, J=1.0, Jzz=1.0, hz=0.0, nup=None):
    bonds = [(i, i + 1, J, Jzz) for i in range(L - 1)]
    H = _sz_sector_hamiltonian(L, bonds, hz, nup)
    if H.shape[0] <= 64:
        return float(np.linalg.eigvalsh(H.toarray())[0])
    return float(spla.eigsh(H, k=1, which="SA", tol=1e-14)[0][0])


def j1j2_ground_energy(L, J1=1.0, J2=0.5, nup=None):
    bonds = [(i, i + 1, J1, J1) for i in range(L - 1)] + [(i, i + 2, J2, J2) for i in range(L - 2)]
    H = _sz_sector_hamiltonian(L, bonds, 0.0, nup)
    if H.shape[0] <= 64:
        return float(np.linalg.eigvalsh(H.toarray())[0])
    return float(spla.eigsh(H, k=1, which="SA", tol=1e-14)[0][0])


def xx_free_fermion_energy(L, J=1.0):
    """Open XX chain 2J(s+s- + h.c.) = hopping t = 2J after Jordan-Wigner;
    single-particle energies 2t cos(k pi/(L+1)); E0 = sum of the negative ones."""
    t = 2.0 * J
    eps = 2.0 * t * np.cos(np.arange(1, L + 1) * np.pi / (L + 1))
    return float(eps[eps < 0].sum())


def tfi_terms(L, h):
    """H = -sum Z_i Z_{i+1} - sum h_i X_i (Pauli matrices)."""
    terms = [(-1.0, {i: SZ, i + 1: SZ}) for i in range(1, L)]
    terms += [(-float(h[i - 1]), {i: SX}) for i in range(1, L + 1)]
    return terms


# -------------------------------------------------- spinful fermions (d=4)
# Local basis index = 2*n_up + n_dn (Julia kron(up, dn): up is the slow index),
# the layout of spinal_fermion_site_ops_dense (utilities/fermion_siteops.jl:64-85).
_a = np.array([[0.0, 1.0], [0.0, 0.0]])       # annihilates the occupied state 1
_n = np.diag([0.0, 1.0])
_p = np.diag([1.0, -1.0])                      # parity (-s_Z)
A_UP = np.kron(_a, I2)
A_DN = np.kron(_p, _a)                         # JW through the up mode of the same site
P4 = np.kron(_p, _p)
N_UPDN = np.kron(_n, _n)
N_TOT = np.kron(_n, I2) + np.kron(I2, _n)


def fermion_product(ops):
    """Product of fermion operators c_{site} given as (site, local matrix);
    each carries the parity string over the sites before it.  Returns the
    per-site local matrices of the product (sites commute after JW)."""
    locs = {}
    for site, m in ops:
        for j in range(1, site):
            locs[j] = locs.get(j, np.eye(4)) @ P4
        locs[site] = locs.get(site, np.eye(4)) @ m
    return locs


def hubbard_ladder_terms(L, J1, J2, U):
    """hubbard_ladder (test/runtests.jl:283-306): U n_up n_dn, -J1 nearest and
    -J2 next-nearest hopping of both spins, plus hermitian conjugates."""
    terms = [(U, {i: N_UPDN}) for i in range(1, L + 1)]
    for (dist, J) in ((1, J1), (2, J2)):
        for i in range(1, L - dist + 1):
            for a in (A_UP, A_DN):
                terms.append((-J, fermion_product([(i, a.T), (i + dist, a)])))
                terms.append((-J, fermion_product([(i + dist, a.T), (i, a)])))
    return terms


def sum_of_products_mpo(L, d, terms):
    """Exact (uncompressed) FiniteMPO of a sum of product terms: the direct
    sum of bond-dimension-1 MPOs, W_1 = row, W_L = column, bulk diagonal."""
    T = len(terms)
    dt = np.result_type(*[np.asarray(c) for c, _ in terms], np.float64)
    Ws = []
    for i in range(1, L + 1):
        wl = 1 if i == 1 else T
        wr = 1 if i == L else T
        W = np.zeros((wl, d, wr, d), dtype=dt)
        for t, (c, ops) in enumerate(terms):
            m = ops.get(i, np.eye(d))
            if i == 1:
                m = c * m
            W[0 if i == 1 else t, :, 0 if i == L else t, :] += m
        Ws.append(W)
    return Ws


def ground_energy_in_sector(H, psi0):
    """Lowest eigenvalue of H inside the conserved sector that contains the
    product state psi0 (basis states reachable from psi0's support)."""
    n = H.shape[0]
    A = (np.abs(H) > 0)
    seen = np.zeros(n, dtype=bool)
    frontier = np.nonzero(np.abs(psi0) > 0)[0]
    seen[frontier] = True
    while len(frontier):
        nxt = np.nonzero(A[:, frontier].any(axis=1) & ~seen)[0]
        seen[nxt] = True
        frontier = nxt
    idx = np.nonzero(seen)[0]
    return float(np.linalg.eigvalsh(H[np.ix_(idx, idx)])[0])


def exact_evolution(H, psi0, t):
    """exp(t * H) psi0 with the dense matrix exponential (exact_timeevolution
    restated, algorithms/exactdiag.jl:58-61)."""
    return scipy.linalg.expm(t * H) @ psi0


def local_expectation(psi, L, d, site, op):
    O = kron_chain([op if i == site else np.eye(d) for i in range(1, L + 1)])
    return np.vdot(psi, O @ psi) / np.vdot(psi, psi)
