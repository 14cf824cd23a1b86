"""Device DMRG1S / TDVP2 / TDVP1S (finitemptools_gb300.expansion) against the
oracle's restatement with explicit null spaces (oracle/expansion.py), exact
diagonalisation and exact evolution."""

import numpy as np
import pytest

import oracle as O
from oracle import ed
from oracle import expansion as OX
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300.utilities import heisenberg_xxz_mpo, tfi_mpo

pytestmark = pytest.mark.gpu
Z = np.diag([-1.0, 1.0])


def _upload(mps, dtype=None):
    return fm.FiniteMPS([DT.from_numpy(A, dtype=dtype) for A in mps])


def test_dmrg1s_matches_oracle_and_ed():
    L = 8
    rng = np.random.default_rng(2)
    st, _ = O.canonicalize(O.randommps(L, 2, 2, rng), normalize=True)
    h = heisenberg_xxz_mpo()
    env_o = O.environments(h.site_tensors(L), st, schur=True)
    env_g = fm.environments(h, _upload(st))
    tr_o = O.MPSTruncation(16, 1e-12)
    alg = fm.DMRG1S(eig_maxiter=20, eig_tol=1e-12, trunc=fm.MPSTruncation(16, 1e-12),
                    verbosity=0)
    for sweep in range(6):
        Eo, do = OX.dmrg1s_sweep(env_o, tr_o, 20, 1e-12)
        Eg, dg = fm.sweep_(env_g, alg)
        assert len(Eg) == len(Eo)
        assert np.abs(np.asarray(Eg) - np.asarray(Eo)).max() < 1e-8 * abs(Eo[-1])
    assert abs(Eg[-1] - ed.xxz_ground_energy(L)) < 1e-8
    assert fm.bond_dimension(env_g.mps) == O.bond_dimension(env_o.mps)


def test_dmrg1s_capped_expansion_at_saturated_bonds():
    """OptimalExpansion(cap=True) at a bond dimension the chain saturates (D=12 <
    32): no degenerate truncation of [B ; V1 NR], so the device and the oracle
    agree entry for entry and the energy settles."""
    L, D = 10, 12
    rng = np.random.default_rng(5)
    st, _ = O.canonicalize(O.randommps(L, 2, 4, rng), normalize=True)
    h = heisenberg_xxz_mpo()
    env_o = O.environments(h.site_tensors(L), st, schur=True)
    env_g = fm.environments(h, _upload(st))
    tr_o = O.MPSTruncation(D, 1e-12)
    alg = fm.DMRG1S(eig_maxiter=20, eig_tol=1e-12, trunc=fm.MPSTruncation(D, 1e-12),
                    expan=fm.OptimalExpansion(cap=True), verbosity=0)
    for _ in range(6):
        Eo, _ = OX.dmrg1s_sweep(env_o, tr_o, 20, 1e-12, cap=True)
        Eg, _ = fm.sweep_(env_g, alg)
        assert np.abs(np.asarray(Eg) - np.asarray(Eo)).max() < 1e-8 * abs(Eo[-1])
    assert fm.bond_dimension(env_g.mps) == D
    assert abs(Eg[-1] - Eg[-L]) < 1e-9 * abs(Eg[-1])
    assert abs(Eg[-1] - ed.xxz_ground_energy(L)) < 1e-3 * abs(Eg[-1])


def test_ground_state_default_is_dmrg1s():
    L = 6
    rng = np.random.default_rng(4)
    st, _ = O.canonicalize(O.randommps(L, 2, 2, rng), normalize=True)
    Es, delta = fm.ground_state_(_upload(st), heisenberg_xxz_mpo(),
                                 fm.DMRG1S(maxiter=8, eig_maxiter=20, trunc=fm.MPSTruncation(8, 1e-12),
                                           verbosity=0))
    assert abs(Es[-1] - ed.xxz_ground_energy(L)) < 1e-8


@pytest.mark.parametrize("algo", ["tdvp2", "tdvp1s"])
def test_tdvp2_and_tdvp1s_match_oracle(algo):
    L, dt, n = 6, 0.05, 4
    rng = np.random.default_rng(3)
    hs = 1.0 + 0.1 * rng.standard_normal(L)
    h = tfi_mpo(hs)
    if algo == "tdvp2":
        st = O.prodmps([np.array([1.0, 0.0]) if i % 2 else np.array([0.6, 0.8]) for i in range(L)],
                       dtype=np.complex128)
    else:
        st = O.prodmps([np.array([0.6, 0.8]) for _ in range(L)], dtype=np.complex128)
    env_o = O.environments([W.astype(complex) for W in h.site_tensors(L)], st, schur=True)
    env_g = fm.environments(h, _upload(st, np.complex128))
    tr = fm.MPSTruncation(16, 1e-12)
    for _ in range(n):
        if algo == "tdvp2":
            OX.tdvp2_sweep(env_o, -1j * dt, O.MPSTruncation(16, 1e-12), exptol=1e-12)
            fm.sweep_(env_g, fm.TDVP2(stepsize=-1j * dt, exptol=1e-12, trunc=tr, krylovdim=30))
        else:
            OX.tdvp1s_sweep(env_o, -1j * dt, O.MPSTruncation(16, 1e-12), exptol=1e-12)
            fm.sweep_(env_g, fm.TDVP1S(stepsize=-1j * dt, exptol=1e-12, trunc=tr, krylovdim=30))
    og = [float(np.real(fm.expectation_local(env_g.mps, i, Z))) for i in range(1, L + 1)]
    oo = [O.single_site_expectation(env_o.mps, i, Z).real for i in range(1, L + 1)]
    assert np.abs(np.array(og) - np.array(oo)).max() < 1e-8
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    psiT = ed.exact_evolution(H, O.mps_to_dense(st), -1j * dt * n)
    ex = [ed.local_expectation(psiT, L, 2, i, Z).real for i in range(1, L + 1)]
    assert np.abs(np.array(og) - np.array(ex)).max() < (1e-4 if algo == "tdvp2" else 1e-3)
