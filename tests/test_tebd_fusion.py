"""fuse_gates (circuit/gate_fusion.jl:357-400) on the host: the fused circuit applies
the same operator (checked on dense state vectors through the oracle's dense_apply), with
the gates the reference's absorption order leaves.  The TEBD stepper's step count."""

import numpy as np
import pytest

import finitemptools_gb300 as fm
from finitemptools_gb300.tebd import QuantumCircuit, QuantumGate
from oracle.tebd import dense_apply


def unitary(rng, n):
    q, r = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def apply_dense(circuit, psi, L, d):
    dims = [d] * L
    for g in circuit:
        psi = dense_apply(psi, L, dims, list(g.positions), g.matrix())
    return psi


def test_fuse_small_cases_follow_the_absorption_order():
    """[A(1), B(1,2), C(2,3)] -> [B A on (1,2), C on (2,3)]: A joins B in the pass over the
    adjoint circuit; B A and C overlap without containing each other, so both stay.
    [B(1,2), A(1)] -> one gate A B on (1,2)."""
    rng = np.random.default_rng(1)
    A, B, C = unitary(rng, 2), unitary(rng, 4), unitary(rng, 4)
    f = fm.fuse_gates(QuantumCircuit([QuantumGate(1, A), QuantumGate((1, 2), B),
                                      QuantumGate((2, 3), C)]))
    assert [g.positions for g in f] == [(1, 2), (2, 3)]
    assert np.allclose(f[0].matrix(), B @ np.kron(np.eye(2), A))
    assert np.allclose(f[1].matrix(), C)
    f2 = fm.fuse_gates(QuantumCircuit([QuantumGate((1, 2), B), QuantumGate(1, A)]))
    assert [g.positions for g in f2] == [(1, 2)]
    assert np.allclose(f2[0].matrix(), np.kron(np.eye(2), A) @ B)
    # no gate contains the sites of A(3): it stays
    f3 = fm.fuse_gates(QuantumCircuit([QuantumGate((1, 2), B), QuantumGate(3, A)]))
    assert [g.positions for g in f3] == [(1, 2), (3,)]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_fuse_random_circuit_keeps_the_operator(seed):
    rng = np.random.default_rng(seed)
    L, d = 6, 2
    gates = []
    for _ in range(30):
        n = int(rng.integers(1, 4))
        start = int(rng.integers(1, L - n + 2))
        pos = list(range(start, start + n))
        if n > 1 and rng.random() < 0.5:
            pos = pos[::-1]                      # unsorted positions, permuted on construction
        gates.append(QuantumGate(tuple(pos), unitary(rng, d ** n)))
    circ = QuantumCircuit(gates)
    fused = fm.fuse_gates(circ)
    assert 0 < len(fused) < len(circ)
    for _ in range(3):
        psi = rng.standard_normal(d ** L) + 1j * rng.standard_normal(d ** L)
        a = apply_dense(circ, psi, L, d)
        b = apply_dense(fused, psi, L, d)
        assert np.linalg.norm(a - b) < 1e-12 * np.linalg.norm(a)


def test_fuse_trotter_circuit_merges_the_half_steps():
    """A second-order Trotter circuit of several steps: consecutive half-step gates on the
    same bond join, the operator is unchanged."""
    rng = np.random.default_rng(5)
    L, d = 6, 2
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    Z = np.diag([1.0, -1.0])
    bonds = {(i, i + 1): -np.kron(Z, Z) for i in range(1, L)}
    sites = {i: -0.7 * X for i in range(1, L + 1)}
    circ = fm.trotter_propagator(L, [d] * L, bonds, sites, tspan=(0.0, -0.3j), order=2,
                                 stepsize=0.05)
    fused = fm.fuse_gates(circ)
    assert len(fused) < len(circ)
    psi = rng.standard_normal(d ** L) + 1j * rng.standard_normal(d ** L)
    a = apply_dense(circ, psi, L, d)
    b = apply_dense(fused, psi, L, d)
    assert np.linalg.norm(a - b) < 1e-12 * np.linalg.norm(a)


def test_tebd_stepper_step_count():
    """compute_step_size / TEBDStepper (algorithms/timeevo.jl:3-33): the span is cut into
    round(|span / stepsize|) steps, at least one, and the stepsize adjusted to divide it."""
    st = fm.TEBDStepper(stepsize=0.03, tspan=(0.0, 0.1))
    assert st.n == 3 and abs(st.stepsize - 0.1 / 3) < 1e-15 and st.delta == 0.1
    st = fm.TEBDStepper(stepsize=1.0, tspan=(0.0, 0.2))
    assert st.n == 1 and st.stepsize == 0.2
    st = fm.TEBDStepper(stepsize=-0.05j)
    assert st.n == 1 and st.tspan == (0.0, -0.05j)


def test_homogeneous_cache_refuses_time_dependent_terms():
    """HomogeousTEBDCache takes a constant Hamiltonian only (timeevo.jl:90 throws
    ArgumentError("const hamiltonian expected.")): a term given as a function of t is
    refused instead of being frozen at the first step."""
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    ZZ = np.kron(np.diag([-1.0, 1.0]), np.diag([-1.0, 1.0]))
    L = 4
    stepper = fm.TEBDStepper(stepsize=0.05, tspan=(0.0, 0.2), order=2)
    bonds = {(i, i + 1): -ZZ for i in range(1, L)}
    with pytest.raises(ValueError, match="const hamiltonian expected"):
        fm.HomogeneousTEBDCache(L, [2] * L, bonds, {1: (lambda t: t * X)}, stepper)
    with pytest.raises(ValueError, match="const hamiltonian expected"):
        fm.HomogeneousTEBDCache(L, [2] * L, {(1, 2): (lambda t: -ZZ)}, {}, stepper)
    cache = fm.HomogeneousTEBDCache(L, [2] * L, bonds, {1: -0.5 * X}, stepper)
    assert len(cache.circuit) > 0


def test_time_dependent_trotter_and_inhomogeneous_cache():
    """Bond and site terms as functions of t (the reference takes each second-order step's
    terms at its midpoint, tebd.jl:99-119): constant functions give the constant circuit
    bit for bit, and a ramped field h(t) = h0 + a t follows the time-ordered evolution
    (a product of 4000 midpoint exponentials) to the Trotter error.  The inhomogeneous
    cache is the fused circuit of the whole span."""
    import scipy.linalg
    L, d = 5, 2
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    Z = np.diag([1.0, -1.0])
    bonds = {(i, i + 1): -np.kron(Z, Z) for i in range(1, L)}
    c0 = fm.trotter_propagator(L, [d] * L, bonds, {i: -0.7 * X for i in range(1, L + 1)},
                               tspan=(0.0, 0.2), order=2, stepsize=0.05)
    c1 = fm.trotter_propagator(L, [d] * L, bonds,
                               {i: (lambda t: -0.7 * X) for i in range(1, L + 1)},
                               tspan=(0.0, 0.2), order=2, stepsize=0.05)
    assert len(c0) == len(c1)
    assert all(a.positions == b.positions and np.array_equal(a.op, b.op) for a, b in zip(c0, c1))

    def field(t):
        return -(0.7 + 1.5 * t) * X

    sites = {i: field for i in range(1, L + 1)}
    T = 0.4
    stepper = fm.TEBDStepper(stepsize=0.01, tspan=(0.0, T), order=2)
    cache = fm.InhomogeneousTEBDCache(L, [d] * L, bonds, sites, stepper)
    circ = fm.trotter_propagator(L, [d] * L, bonds, sites, tspan=(0.0, T), order=2,
                                 stepsize=0.01)
    assert len(cache.circuit) < len(circ)

    def dense_H(t):
        H = np.zeros((d ** L, d ** L))
        for i in range(1, L):
            H += kron_sites(L, {i: -Z, i + 1: Z})
        for i in range(1, L + 1):
            H += kron_sites(L, {i: field(t)})
        return H

    rng = np.random.default_rng(8)
    psi = rng.standard_normal(d ** L)
    psi /= np.linalg.norm(psi)
    ref = psi.copy()
    n = 4000
    for k in range(n):
        ref = scipy.linalg.expm((T / n) * dense_H((k + 0.5) * T / n)) @ ref
    a = apply_dense(cache.circuit, psi, L, d)
    b = apply_dense(circ, psi, L, d)
    assert np.linalg.norm(a - b) < 1e-12 * np.linalg.norm(b)
    assert np.linalg.norm(a - ref) < 1e-3 * np.linalg.norm(ref)


def kron_sites(L, ops):
    """The operator with ops[i] on site i (1-based), first site fastest."""
    m = np.ones((1, 1))
    for i in range(L, 0, -1):
        m = np.kron(m, ops.get(i, np.eye(2)))
    return m
