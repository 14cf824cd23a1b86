"""CPU pins of the restated DMRG1S / TDVP2 / TDVP1S (oracle/expansion.py):
ground energies against exact diagonalisation and observables against exact
evolution, the reference's own kinds of checks (test/runtests.jl:773-790)."""

import numpy as np

import oracle as O
from oracle import ed
from oracle import expansion as OX
from finitemptools_gb300.utilities import FiniteMPO, heisenberg_xxz_mpo, tfi_mpo

Z = np.diag([-1.0, 1.0])


def test_dmrg1s_grows_bond_and_matches_ed():
    L = 8
    rng = np.random.default_rng(2)
    st, _ = O.canonicalize(O.randommps(L, 2, 2, rng), normalize=True)
    env = O.environments(heisenberg_xxz_mpo().site_tensors(L), st, schur=True)
    tr = O.MPSTruncation(16, 1e-12)
    for _ in range(6):
        Es, _ = OX.dmrg1s_sweep(env, tr, 20, 1e-12)
    assert O.bond_dimension(env.mps) > 2
    assert abs(Es[-1] - ed.xxz_ground_energy(L)) < 1e-8


def _tfi(L, seed):
    rng = np.random.default_rng(seed)
    hs = 1.0 + 0.1 * rng.standard_normal(L)
    return hs, tfi_mpo(hs)


def test_tdvp2_matches_exact_evolution():
    L, dt, n = 6, 0.05, 4
    hs, h = _tfi(L, 3)
    st = O.prodmps([np.array([1.0, 0.0]) if i % 2 else np.array([0.6, 0.8]) for i in range(L)],
                   dtype=np.complex128)
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    psiT = ed.exact_evolution(H, O.mps_to_dense(st), -1j * dt * n)
    env = O.environments([W.astype(complex) for W in h.site_tensors(L)], st, schur=True)
    for _ in range(n):
        OX.tdvp2_sweep(env, -1j * dt, O.MPSTruncation(16, 1e-12), exptol=1e-12)
    obs = [O.single_site_expectation(env.mps, i, Z).real for i in range(1, L + 1)]
    ex = [ed.local_expectation(psiT, L, 2, i, Z).real for i in range(1, L + 1)]
    # second-order splitting error of the two-site integrator at dt = 0.05
    assert np.max(np.abs(np.array(obs) - ex)) < 1e-4


def test_tdvp1s_expands_from_a_product_state():
    L, dt, n = 6, 0.05, 4
    hs, h = _tfi(L, 4)
    st = O.prodmps([np.array([0.6, 0.8]) for _ in range(L)], dtype=np.complex128)
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    psiT = ed.exact_evolution(H, O.mps_to_dense(st), -1j * dt * n)
    env = O.environments([W.astype(complex) for W in h.site_tensors(L)], st, schur=True)
    for _ in range(n):
        OX.tdvp1s_sweep(env, -1j * dt, O.MPSTruncation(16, 1e-12), exptol=1e-12)
    assert O.bond_dimension(env.mps) > 1                  # the expansion grew the bonds
    obs = [O.single_site_expectation(env.mps, i, Z).real for i in range(1, L + 1)]
    ex = [ed.local_expectation(psiT, L, 2, i, Z).real for i in range(1, L + 1)]
    assert np.max(np.abs(np.array(obs) - ex)) < 1e-3
