"""TEBD on the device (finitemptools_gb300.tebd, fmpt_apply_gate) against the
oracle's restatement (oracle/tebd.py), dense gate application and exact
evolution."""

import numpy as np
import pytest

import oracle as O
from oracle import ed
from oracle import tebd as OT
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT

pytestmark = pytest.mark.gpu
Z = np.diag([-1.0, 1.0])
SX = np.array([[0.0, 1.0], [1.0, 0.0]])


def _canonical(L, D, seed, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    mps, s = O.canonicalize(O.randommps(L, 2, D, rng, dtype=dtype), normalize=True)
    s[0] = np.ones(1)
    s[L] = np.ones(1)
    return mps, s


def _upload(mps, s):
    psi = fm.FiniteMPS.from_numpy(mps)
    for i in range(1, len(mps) + 2):
        psi.s[i] = DT.from_numpy(np.asarray(s[i - 1], dtype=np.float64))
    return psi


def _dense(psi):
    return O.mps_to_dense([psi[i].numpy() for i in range(1, len(psi) + 1)])


def _random_unitary(P, rng):
    q, r = np.linalg.qr(rng.standard_normal((P, P)) + 1j * rng.standard_normal((P, P)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("pos", [(3,), (2, 3), (2, 5), (5, 2), (1, 2, 3), (1, 3, 6), (2, 3, 4, 5),
                                 (1, 3, 4, 7), (7, 2, 4, 5)])
def test_gates_match_dense_and_oracle(pos):
    L = 7
    mps, s = _canonical(L, 8, 1)
    rng = np.random.default_rng(len(pos) * 10 + pos[0])
    g = fm.QuantumGate(pos, _random_unitary(2 ** len(pos), rng))
    psi0 = O.mps_to_dense(mps)
    psi = _upload(mps, s)
    errs = fm.apply_(g, psi, trunc=fm.MPSTruncation(1000, 0.0))
    assert len(errs) == 1
    ref = OT.dense_apply(psi0, L, [2] * L, g.positions, g.matrix())
    assert np.abs(_dense(psi) - ref).max() < 1e-12
    mo, so = [A.copy() for A in mps], list(s)
    OT.apply_gate(g.positions, g.matrix(), mo, so, O.MPSTruncation(1000, 0.0))
    for i in range(2, L + 1):      # Schmidt values agree with the oracle's
        assert np.abs(psi.s[i].numpy() - so[i - 1]).max() < 1e-12


@pytest.mark.parametrize("svd,tol", [("gesvd", 1e-10), ("dm", 1e-7)])
def test_trotter_tebd_matches_oracle_and_exact(svd, tol):
    L, T, dt = 10, 0.5, 0.05
    rng = np.random.default_rng(3)
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    bonds = {(i, i + 1): -np.kron(Z, Z) for i in range(1, L)}
    sites = {i: -hs[i - 1] * SX for i in range(1, L + 1)}
    circ = fm.trotter_propagator(L, [2] * L, bonds, sites, tspan=(0.0, -1j * T), order=4,
                                 stepsize=dt)
    st = O.prodmps([np.array([0.6, 0.8])] * L, dtype=np.complex128)
    mps, s = O.canonicalize(st, normalize=True)
    s[0], s[L] = np.ones(1), np.ones(1)
    psi = _upload(mps, s)
    errs = fm.apply_(circ, psi, trunc=fm.MPSTruncation(64, 1e-12), svd=svd)
    assert len(errs) == len(circ)
    OT.apply_circuit([(g.positions, g.matrix()) for g in circ], mps, s,
                     O.MPSTruncation(64, 1e-12))
    got, oref = _dense(psi), O.mps_to_dense(mps)
    assert abs(abs(np.vdot(oref, got)) - 1.0) < tol
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    ref = ed.exact_evolution(H, O.mps_to_dense(st), -1j * T)
    zs = [float(np.real(fm.expectation_local(psi, i, Z))) for i in range(1, L + 1)]
    zr = [ed.local_expectation(ref, L, 2, i, Z).real for i in range(1, L + 1)]
    assert np.abs(np.array(zs) - np.array(zr)).max() < 2e-6


def test_tebd_stepper_fused_circuit():
    """TEBDStepper + HomogeneousTEBDCache + make_step_ (algorithms/timeevo.jl): 8 fused
    second-order steps of -0.05i on TFI L=8.  The device state matches the oracle's
    application of the unfused circuit, with fewer gates, and the exact evolution to the
    Trotter error."""
    L = 8
    rng = np.random.default_rng(9)
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    bonds = {(i, i + 1): -np.kron(Z, Z) for i in range(1, L)}
    sites = {i: -hs[i - 1] * SX for i in range(1, L + 1)}
    stepper = fm.TEBDStepper(stepsize=-0.05j, tspan=(0.0, -0.4j), order=2,
                             trunc=fm.MPSTruncation(64, 1e-12))
    assert stepper.n == 8
    cache = fm.HomogeneousTEBDCache(L, [2] * L, bonds, sites, stepper)
    one = fm.trotter_propagator(L, [2] * L, bonds, sites, tspan=(0.0, -0.05j), order=2,
                                stepsize=-0.05j)
    assert len(cache.circuit) < 8 * len(one)
    st = O.prodmps([np.array([0.6, 0.8])] * L, dtype=np.complex128)
    mps, s = O.canonicalize(st, normalize=True)
    s[0], s[L] = np.ones(1), np.ones(1)
    psi = _upload(mps, s)
    fm.make_step_(cache, psi)
    OT.apply_circuit([(g.positions, g.matrix()) for g in list(one) * 8], mps, s,
                     O.MPSTruncation(64, 1e-12))
    got, oref = _dense(psi), O.mps_to_dense(mps)
    assert abs(abs(np.vdot(oref, got)) - 1.0) < 1e-10
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    ref = ed.exact_evolution(H, O.mps_to_dense(st), -0.4j)
    ref = ref / np.linalg.norm(ref)
    assert abs(abs(np.vdot(ref, got)) - 1.0) < 1e-4


def test_uninitialised_svectors_are_canonicalised_and_dtype_checked():
    L = 5
    rng = np.random.default_rng(4)
    st = O.randommps(L, 2, 4, rng)
    psi = fm.FiniteMPS.from_numpy(st)
    g = fm.QuantumGate((2, 3), _random_unitary(4, rng))
    with pytest.raises(TypeError):
        fm.apply_(g, psi)
    gr = fm.QuantumGate((2, 3), np.kron(SX, Z))
    d0 = O.mps_to_dense(st)
    fm.apply_(gr, psi, trunc=fm.MPSTruncation(100, 0.0))
    ref = OT.dense_apply(d0, L, [2] * L, (2, 3), gr.matrix())
    assert np.abs(_dense(psi) - ref).max() < 1e-12


@pytest.mark.parametrize("method", ["gesvdp", "gesvdj"])
@pytest.mark.parametrize("shape,cplx,rank", [((512, 512), True, None), ((300, 700), False, None),
                                             ((1024, 1024), False, None), ((200, 90), True, 40)])
def test_alternative_svd_matches_gesvd(shape, cplx, rank, method):
    """fmpt_set_svd_method(1 / 2): the polar-decomposition and Jacobi SVDs give
    the gesvd singular values (descending) and an exact factorisation.
    Measured for the polar form: 1e-11 relative on full-rank matrices; on a
    rank-deficient matrix its zero singular values come out near 1e-11 sigma_max
    and the others agree to about 1e-8 relative, which is why gesvd stays the
    default."""
    from finitemptools_gb300.auxiliary import stable_tsvd
    rng = np.random.default_rng(sum(shape))
    m, n = shape
    A = rng.standard_normal(shape) + (1j * rng.standard_normal(shape) if cplx else 0)
    if rank is not None:
        A = A[:, :rank] @ rng.standard_normal((rank, n))
    h = fm.default_handle()
    out = {}
    for meth in ("gesvd", method):
        h.set_svd_method(meth)
        u, s, vt, _ = stable_tsvd(DT.from_numpy(A), m, n)
        out[meth] = (u.numpy(), s.numpy(), vt.numpy())
    h.set_svd_method("gesvd")
    u, s, vt = out[method]
    s0 = out["gesvd"][1]
    scale = max(1.0, np.abs(s0).max())
    tol = 1e-11 if rank is None else 1e-9
    assert s.shape == s0.shape
    assert np.all(np.diff(s) <= 1e-12 * scale)
    assert np.abs(s - s0).max() < tol * scale
    assert np.abs((u * s[None, :]) @ vt - A).max() < tol * scale
    keep = s > 1e-8 * scale
    uk, vk = u[:, keep], vt[keep, :]
    assert np.abs(uk.conj().T @ uk - np.eye(uk.shape[1])).max() < 1e-11
    assert np.abs(vk @ vk.conj().T - np.eye(vk.shape[0])).max() < 1e-11
