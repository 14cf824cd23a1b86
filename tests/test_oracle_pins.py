"""Pins of the CPU oracle against the reference's own checks.

The reference ships no golden vectors; its tests compare DMRG energies with
exact diagonalisation to 1e-8 (test/runtests.jl:773-778, do_dmrg :413-421:
5 sweeps of DMRG2() with default parameters), TDVP observables with exact
time evolution to 1e-4 (:786-790, stepsize -0.01im, 50 sweeps) and <H> from
an MPO with a dense contraction to 1e-8 (:765-770).  The same checks are
restated here for the oracle on dense models.
"""

import numpy as np
import pytest

import oracle as O
from oracle import ed
from finitemptools_gb300.utilities import (FiniteMPO, heisenberg_xxz_mpo,
                                           j1j2_heisenberg_mpo, tfi_mpo)


def _do_dmrg(env, sweeps=5, **kw):
    Es = None
    for _ in range(sweeps):
        Es, delta = O.dmrg2_sweep(env, **kw)
    return Es[-1], delta


@pytest.mark.parametrize("L", [5, 6])
def test_dmrg2_hubbard_ladder_equals_ed(L):
    terms = ed.hubbard_ladder_terms(L, 1.0, 1.2, 1.37)        # test_ground_state :423-451
    H = ed.dense_from_terms(L, 4, terms)
    mpo = ed.sum_of_products_mpo(L, 4, terms)
    rng = np.random.default_rng(100 + L)
    st, _ = O.canonicalize(O.randommps(L, 4, 8, rng), normalize=True)
    E, _ = _do_dmrg(O.environments(mpo, st))
    assert abs(E - np.linalg.eigvalsh(H)[0]) < 1e-8


@pytest.mark.parametrize("L", [5, 6])
def test_dmrg2_mpohamiltonian_vs_finitempo_vs_ed(L):
    """test_ground_state_2 (:453-492) restated: Schur-form environments and
    the dense FiniteMPO(h, L) embedding give the ED energy."""
    h = heisenberg_xxz_mpo(1.0, 0.8, 0.37)
    H = ed.dense_from_terms(L, 2, ed.xxz_terms(L, 1.0, 0.8, 0.37))
    E0 = np.linalg.eigvalsh(H)[0]
    rng = np.random.default_rng(7)
    st, _ = O.canonicalize(O.randommps(L, 2, 4, rng), normalize=True)
    E1, _ = _do_dmrg(O.environments(FiniteMPO(h, L), st))
    E2, _ = _do_dmrg(O.environments(h.site_tensors(L), st, schur=True))
    assert abs(E1 - E0) < 1e-8
    assert abs(E2 - E0) < 1e-8


def test_dmrg1_equals_ed():
    L = 6
    H = ed.dense_from_terms(L, 2, ed.xxz_terms(L, 1.0, 1.0, 0.2))
    rng = np.random.default_rng(9)
    st, _ = O.canonicalize(O.randommps(L, 2, 8, rng), normalize=True)
    env = O.environments(FiniteMPO(heisenberg_xxz_mpo(1.0, 1.0, 0.2), L), st)
    for _ in range(5):
        Es, _ = O.dmrg1_sweep(env, D=50)
    assert abs(Es[-1] - np.linalg.eigvalsh(H)[0]) < 1e-8


def test_expectation_values():
    """expectation values (:765-770): <H> from the MPO environment chain
    equals the dense contraction."""
    L = 7
    rng = np.random.default_rng(11)
    st, _ = O.canonicalize(O.randommps(L, 2, 6, rng), normalize=True)
    h = j1j2_heisenberg_mpo(1.0, 0.5)
    psi = O.mps_to_dense(st)
    Hd = O.mpo_to_dense(FiniteMPO(h, L))
    ref = np.vdot(psi, Hd @ psi)
    assert abs(O.expectation_mpo(st, FiniteMPO(h, L)) - ref) < 1e-8
    assert abs(O.expectation_mpo(st, h.site_tensors(L), schur=True) - ref) < 1e-8


def test_tdvp1_hubbard_equals_exact_evolution():
    """test_tdvp (:550-594) restated for TDVP1 on the dense Hubbard ladder:
    <n_i> after 50 steps of stepsize -0.01im agrees with exp(-iHt) to 1e-4."""
    L, dt, n = 4, 0.01, 50
    terms = ed.hubbard_ladder_terms(L, 1.0, 1.2, 0.7)
    H = ed.dense_from_terms(L, 4, terms)
    mpo = [W.astype(complex) for W in ed.sum_of_products_mpo(L, 4, terms)]
    st = O.prodmps([np.eye(4)[0] if i % 2 == 0 else np.eye(4)[3] for i in range(L)],
                   dtype=np.complex128)                     # initial_state_dense :332-338
    psiT = ed.exact_evolution(H, O.mps_to_dense(st), -1j * dt * n)
    env = O.environments(mpo, st)
    for _ in range(n):
        O.tdvp1_sweep(env, -1j * dt, D=50, exptol=1e-8)
    obs = [O.single_site_expectation(env.mps, i, ed.N_TOT).real for i in range(1, L + 1)]
    ex = [ed.local_expectation(psiT, L, 4, i, ed.N_TOT).real for i in range(1, L + 1)]
    assert np.max(np.abs(np.array(obs) - ex)) < 1e-4


def test_mpo_builders_match_terms():
    L = 6
    for h, terms in ((heisenberg_xxz_mpo(1.0, 0.7, 0.3), ed.xxz_terms(L, 1.0, 0.7, 0.3)),):
        assert np.abs(O.mpo_to_dense(FiniteMPO(h, L)) - ed.dense_from_terms(L, 2, terms)).max() < 1e-13
    hs = np.linspace(0.9, 1.1, L)
    assert np.abs(O.mpo_to_dense(FiniteMPO(tfi_mpo(hs), L))
                  - ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))).max() < 1e-13
    # J1-J2 against the sector Hamiltonian's spectrum
    Hd = O.mpo_to_dense(FiniteMPO(j1j2_heisenberg_mpo(1.0, 0.5), L))
    assert abs(np.linalg.eigvalsh(Hd)[0] - ed.j1j2_ground_energy(L, 1.0, 0.5)) < 1e-10


def test_xx_free_fermion_closed_form():
    L = 10
    H = ed.dense_from_terms(L, 2, ed.xxz_terms(L, 1.0, 0.0, 0.0))
    assert abs(np.linalg.eigvalsh(H)[0] - ed.xx_free_fermion_energy(L)) < 1e-10


def test_lanczos_restatement_early_exit():
    """simple_lanczos.jl:86-89: beta < btol after the first step returns the
    Rayleigh quotient and the normalised start vector."""
    A = np.diag([1.0, 2.0, 3.0])
    v = np.array([0.0, 2.0, 0.0])
    E, vec, info, k = O.simple_lanczos_solver(lambda x: A @ x, v, 10, 1e-12)
    assert k == 1 and E == 2.0 and np.allclose(vec, [0, 1, 0])


def test_truncation_semantics():
    s = np.array([1.0, 0.5, 1e-3, 1e-9, 1e-12])
    k, err = O.mps_truncate(s, O.MPSTruncation(10, 1e-8))
    assert k == 3 and abs(err - np.linalg.norm(s[3:])) < 1e-20
    k, err = O.mps_truncate(s, O.MPSTruncation(2, 1e-8))
    assert k == 2 and abs(err - np.linalg.norm(s[2:])) < 1e-18
