"""CPU pins of the restated TEBD gate application (oracle/tebd.py) and of the
product's host-side Trotter circuit builder (finitemptools_gb300.tebd, no GPU
needed to build gates): exact gate action against dense application for 1- to
4-site gates at neighbouring and distant positions, and the order-2 / order-4
Trotter circuits against exact evolution, the reference's test_tebd check
(test/runtests.jl:596-633)."""

import numpy as np
import pytest

import oracle as O
from oracle import ed
from oracle import tebd as OT
from finitemptools_gb300.tebd import QuantumGate, trotter_propagator

Z = np.diag([-1.0, 1.0])
SX = np.array([[0.0, 1.0], [1.0, 0.0]])


def _canonical(L, D, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    mps, s = O.canonicalize(O.randommps(L, 2, D, rng, dtype=dtype), normalize=True)
    s[0] = np.ones(1)
    s[L] = np.ones(1)
    return mps, s


def _random_unitary(P, rng):
    q, r = np.linalg.qr(rng.standard_normal((P, P)) + 1j * rng.standard_normal((P, P)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("pos", [(3,), (2, 3), (2, 5), (5, 2), (1, 2, 3), (1, 3, 6), (2, 3, 4, 5),
                                 (1, 3, 4, 7), (7, 2, 4, 5)])
def test_gate_application_is_exact_without_truncation(pos):
    L = 7
    mps, s = _canonical(L, 8, 1)
    rng = np.random.default_rng(len(pos) * 10 + pos[0])
    P = 2 ** len(pos)
    g = QuantumGate(pos, _random_unitary(P, rng))
    psi0 = O.mps_to_dense(mps)
    OT.apply_gate(g.positions, g.matrix(), mps, s, O.MPSTruncation(1000, 0.0))
    ref = OT.dense_apply(psi0, L, [2] * L, g.positions, g.matrix())
    assert np.abs(O.mps_to_dense(mps) - ref).max() < 1e-12
    # the tensors stay right-canonical and the s-vectors are Schmidt values
    for i in range(1, L):
        B = mps[i]
        M = B.reshape(B.shape[0], -1, order="F")
        assert np.abs(M @ M.conj().T - np.eye(M.shape[0])).max() < 1e-12


def test_gate_position_sorting_permutes_the_operator():
    rng = np.random.default_rng(2)
    U = _random_unitary(4, rng)
    g = QuantumGate((5, 2), U)
    assert g.positions == (2, 5)
    psi = rng.standard_normal(2 ** 6) + 0j
    a = OT.dense_apply(psi, 6, [2] * 6, (5, 2), U)
    b = OT.dense_apply(psi, 6, [2] * 6, g.positions, g.matrix())
    assert np.abs(a - b).max() < 1e-14


@pytest.mark.parametrize("order,tol", [(2, 2e-4), (4, 2e-7)])
def test_trotter_circuit_matches_exact_evolution(order, tol):
    L, T, dt = 8, 0.5, 0.05
    rng = np.random.default_rng(3)
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    bonds = {(i, i + 1): -np.kron(Z, Z) for i in range(1, L)}
    sites = {i: -hs[i - 1] * SX for i in range(1, L + 1)}
    circ = trotter_propagator(L, [2] * L, bonds, sites, tspan=(0.0, -1j * T), order=order,
                              stepsize=dt)
    st = O.prodmps([np.array([0.6, 0.8])] * L, dtype=np.complex128)
    mps, s = O.canonicalize(st, normalize=True)
    s[0], s[L] = np.ones(1), np.ones(1)
    OT.apply_circuit([(g.positions, g.matrix()) for g in circ], mps, s,
                     O.MPSTruncation(64, 1e-12))
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    ref = ed.exact_evolution(H, O.mps_to_dense(st), -1j * T)
    got = O.mps_to_dense(mps)
    assert abs(abs(np.vdot(ref, got)) - 1.0) < tol
    zs = [ed.local_expectation(got, L, 2, i, Z).real for i in range(1, L + 1)]
    zr = [ed.local_expectation(ref, L, 2, i, Z).real for i in range(1, L + 1)]
    assert np.abs(np.array(zs) - np.array(zr)).max() < 10 * tol
