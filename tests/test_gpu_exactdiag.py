"""Exact diagonalisation and exact time evolution through the device ac_prime
(finitemptools_gb300.exactdiag, fmpt_eigsolve) against dense linear algebra,
the ED fixture and the oracle's restatement (oracle/exactdiag.py)."""

import json
import os

import numpy as np
import pytest

import oracle as O
from oracle import ed
from oracle import exactdiag as OX
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300.utilities import FiniteMPO, heisenberg_xxz_mpo, tfi_mpo

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.diag([-1.0, 1.0])


def _dense(st):
    return O.mps_to_dense([st[i].numpy() for i in range(1, len(st) + 1)])


@pytest.mark.parametrize("form", ["finitempo", "schur"])
def test_ed_lowest_states_match_dense(form):
    L = 10
    rng = np.random.default_rng(3)
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    h = tfi_mpo(hs)
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    E = np.linalg.eigvalsh(H)
    if form == "finitempo":
        vals, states = fm.exact_diagonalization(FiniteMPO(h, L), num=4,
                                                rng=np.random.default_rng(0))
    else:
        vals, states = fm.exact_diagonalization(h, len=L, num=4, rng=np.random.default_rng(0))
    assert np.abs(np.asarray(vals) - E[:4]).max() < 1e-10
    vs = np.stack([_dense(st) for st in states], axis=1)
    assert np.abs(vs.T @ vs - np.eye(4)).max() < 1e-10
    for i in range(4):
        assert np.linalg.norm(H @ vs[:, i] - vals[i] * vs[:, i]) < 1e-8
    # the states are FiniteMPS in mixed canonical form: local observables work
    st = states[0].to_finite_mps()
    z = fm.expectation_local(st, 3, Z)
    assert abs(z - ed.local_expectation(vs[:, 0], L, 2, 3, Z)) < 1e-10


def test_ed_xxz_L20_matches_fixture():
    with open(os.path.join(HERE, "golden", "exact_energies.json")) as f:
        e_ref = json.load(f)["xxz_L20_J1_Jzz1_hz0"]
    vals, states = fm.exact_diagonalization(heisenberg_xxz_mpo(), len=20, num=1,
                                            rng=np.random.default_rng(1), tol=1e-10)
    assert states[0].center == 10 and states[0][10].shape == (512, 2, 1024)
    assert abs(vals[0] - e_ref) < 1e-9 * abs(e_ref)


def test_eigsolve_highest_and_projected():
    """which='LR' and an operator composed with _project!: projecting out the
    lowest eigenvector leaves the next ones."""
    rng = np.random.default_rng(4)
    L = 8
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    psi = fm.ExactFiniteMPS.random([2] * L, rng=rng)
    left, right, Wc = fm.init_h_center(FiniteMPO(tfi_mpo(hs), L), psi)
    op = fm.HeffOp("ac", left, right, W1=Wc)
    E = np.linalg.eigvalsh(ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs)))
    x0 = psi[psi.center]
    hi, _, info = op.eigsolve(x0, num=2, which="LR")
    assert info["converged"] >= 2
    assert np.abs(np.asarray(hi) - E[::-1][:2]).max() < 1e-10
    lo, vecs, _ = op.eigsolve(x0, num=1)
    op.set_projectors([vecs[0]])
    x1 = fm.project_(x0.copy(), [vecs[0]])
    nxt, _, _ = op.eigsolve(x1, num=2)
    assert np.abs(np.asarray(nxt) - E[1:3]).max() < 1e-9


def test_exact_time_evolution_non_hermitian():
    """ishermitian=False (the reference's Arnoldi driver) on a non-Hermitian H: TFI with
    complex fields h_i + i g_i.  Time evolution against the dense matrix exponential, for a
    real and an imaginary time; the two eigenvalues of lowest real part against the dense
    spectrum, with the returned states' residuals."""
    from finitemptools_gb300.utilities import MPOHamiltonian, SchurMPOTensor, spin_half_matrices
    L = 8
    rng = np.random.default_rng(11)
    hc = 1.0 + 0.2 * rng.standard_normal(L) + 0.3j * rng.standard_normal(L)
    p = spin_half_matrices()
    data = []
    for hi in hc:
        O_ = [[0] * 3 for _ in range(3)]
        O_[0][0] = np.eye(2)
        O_[0][1] = -p["z"]
        O_[0][2] = -hi * p["x"]
        O_[1][2] = p["z"]
        O_[2][2] = np.eye(2)
        data.append(SchurMPOTensor(O_))
    mpo = FiniteMPO(MPOHamiltonian(data), L)
    terms = [(-1.0, {i: ed.SZ, i + 1: ed.SZ}) for i in range(1, L)]
    terms += [(-hc[i - 1], {i: ed.SX}) for i in range(1, L + 1)]
    H = ed.dense_from_terms(L, 2, terms)
    assert np.abs(H - H.conj().T).max() > 0.1
    st = O.randommps(L, 2, 3, rng, dtype=np.complex128)
    ex = fm.ExactFiniteMPS.from_mps(fm.FiniteMPS.from_numpy(st))
    for t in (0.3, -0.4j):
        out = fm.exact_timeevolution(mpo, t, ex, ishermitian=False)
        ref = ed.exact_evolution(H, O.mps_to_dense(st), t)
        assert np.linalg.norm(_dense(out) - ref) < 1e-9 * np.linalg.norm(ref)
    vals, states = fm.exact_diagonalization(mpo, ishermitian=False, num=2, which="SR",
                                            rng=np.random.default_rng(12))
    ev = np.linalg.eigvals(H)
    ev = ev[np.argsort(ev.real, kind="stable")][:2]
    assert np.abs(np.array(vals) - ev).max() < 1e-8, (vals, ev)
    for lam, st_ in zip(vals, states):
        v = _dense(st_)
        assert np.linalg.norm(H @ v - lam * v) < 1e-6 * np.linalg.norm(v)


def test_exact_mps_and_time_evolution():
    L, t = 9, -0.4j
    rng = np.random.default_rng(5)
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    h = tfi_mpo(hs)
    st = O.randommps(L, 2, 3, rng, dtype=np.complex128)
    psi = fm.FiniteMPS.from_numpy(st)
    ex = fm.ExactFiniteMPS.from_mps(psi)
    ex_o, mid = OX.exact_mps_from(st)
    assert ex.center == mid
    assert np.abs(_dense(ex) - O.mps_to_dense(st)).max() < 1e-13
    out = fm.exact_timeevolution(FiniteMPO(h, L), t, ex)
    ref = ed.exact_evolution(ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs)),
                             O.mps_to_dense(st), t)
    assert np.abs(_dense(out) - ref).max() < 1e-9
    ref_o = OX.exact_timeevolution(FiniteMPO(h, L), t, ex_o, mid)
    assert np.abs(_dense(out) - O.mps_to_dense(ref_o)).max() < 1e-9
    # a real state with a complex time is promoted
    ex_r = fm.ExactFiniteMPS.from_mps(fm.FiniteMPS.from_numpy(O.randommps(L, 2, 2, rng)))
    out_r = fm.exact_timeevolution(FiniteMPO(h, L), -0.1j, ex_r)
    assert out_r.dtype == np.complex128
