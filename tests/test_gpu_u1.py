"""Parity of the U(1) block-sparse device path (grouped persistent engine)
against the oracle's block-sparse restatement, the dense FP64 device path and
exact diagonalisation.

Bar: the plain FP64 bar of the dense path -- H_eff*x and environment updates
within 1e-12 relative of the oracle (they reach ~1e-15), exact zeros outside
the allowed charge blocks, split factors within 1e-12, sweep energies within
1e-10 of exact diagonalisation in the Sz sector.
"""

import numpy as np
import pytest

import oracle as O
from oracle import u1 as OU
from oracle.ed import xxz_ground_energy
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300.u1 import (U1FiniteMPS, U1Space, u1_pack2, u1_right_canonicalize_,
                                    u1_unpack2)
from finitemptools_gb300.utilities import heisenberg_xxz_mpo, j1j2_heisenberg_mpo

pytestmark = pytest.mark.gpu
QP = (0, 1)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def sp(leg):
    return U1Space(leg.items())


def _bond(L, N, D, site, seed, mpo=None):
    rng = np.random.default_rng(seed)
    Ws = (mpo or heisenberg_xxz_mpo(1.0, 0.7, 0.3)).site_tensors(L)
    qw = OU.channel_charges(Ws, list(QP))
    mps, legs = OU.random_u1_state(L, N, D, list(QP), rng)
    w = Ws[0].shape[0]
    Vl, Vr = legs[site - 1], legs[site + 1]
    Lm = rng.standard_normal((Vl.dim, w, Vl.dim)) * OU.allowed_env(Vl, qw[site - 1])
    Rm = rng.standard_normal((Vr.dim, w, Vr.dim)) * OU.allowed_env(Vr, qw[site + 1])
    return Ws, qw, mps, legs, Lm, Rm


@pytest.mark.parametrize("L,N,D,site", [(6, 3, 4, 3), (10, 5, 20, 5), (12, 4, 33, 2),
                                        (16, 8, 96, 8), (24, 12, 300, 12)])
def test_u1_ac2_apply(L, N, D, site):
    Ws, qw, mps, legs, Lm, Rm = _bond(L, N, D, site, L + D)
    Vl, Vr = legs[site - 1], legs[site + 1]
    W1, W2 = Ws[site - 1], Ws[site]
    X = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
    ref = O.ac2_prime(X, W1, W2, Lm, Rm)
    dL, dR = DT.from_numpy(Lm), DT.from_numpy(Rm)
    op = fm.U1HeffOp(dL, dR, W1, W2, sp(Vl), sp(Vr), QP, QP, qw[site - 1], qw[site],
                     qw[site + 1])
    x = DT.from_numpy(OU.pack2(X, Vl, Vr, list(QP), list(QP)))
    assert op.n == x.size
    y = op(x).numpy()
    assert rel(y, OU.pack2(ref, Vl, Vr, list(QP), list(QP))) < 1e-13
    # the dense FP64 device path on the same charge-sorted tensors
    yd = fm.ac2_prime(DT.from_numpy(X), W1, W2, dL, dR).numpy()
    assert rel(y, OU.pack2(yd, Vl, Vr, list(QP), list(QP))) < 1e-13
    # repeated application is bit-identical (fixed summation order)
    assert np.array_equal(op(x).numpy(), y)
    assert op.flops() > 0


@pytest.mark.parametrize("L,N,D,site", [(10, 5, 20, 5), (16, 8, 96, 8), (24, 12, 300, 12)])
def test_u1_tile_variants_identical(L, N, D, site):
    """Every grouped-kernel variant (32x32 or 64x64 tiles, each with both block
    schedules) sums every output in the same order: forced any way, H_eff*x and the
    environment update agree bit for bit; the autotuner caches a decision for large
    programs."""
    Ws, qw, mps, legs, Lm, Rm = _bond(L, N, D, site, 5 * L + D)
    Vl, Vm, Vr = legs[site - 1], legs[site], legs[site + 1]
    W1, W2 = Ws[site - 1], Ws[site]
    X = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
    dL, dR = DT.from_numpy(Lm), DT.from_numpy(Rm)
    x = DT.from_numpy(OU.pack2(X, Vl, Vr, list(QP), list(QP)))
    A = DT.from_numpy(mps[site - 1])
    h = dL.h
    ys, es = [], []
    try:
        for mode, tile in ((1, 32), (2, 64), (3, 32), (4, 64)):
            h.set_tuning(mode)
            op = fm.U1HeffOp(dL, dR, W1, W2, sp(Vl), sp(Vr), QP, QP, qw[site - 1], qw[site],
                             qw[site + 1])
            assert op.tile() == tile
            ys.append(op(x).numpy())
            es.append(fm.u1_updateleft(dL, A, W1, A, sp(Vl), sp(Vm), QP, qw[site - 1],
                                       qw[site]).numpy())
        h.set_tuning(0)
        op = fm.U1HeffOp(dL, dR, W1, W2, sp(Vl), sp(Vr), QP, QP, qw[site - 1], qw[site],
                         qw[site + 1])
        y_auto = op(x).numpy()
        if op.flops() >= 2e7:
            assert h.tuning_info()[0] >= 1
    finally:
        h.set_tuning(0)
    assert all(np.array_equal(ys[0], y) for y in ys[1:]) and np.array_equal(y_auto, ys[0])
    assert all(np.array_equal(es[0], e) for e in es[1:])
    assert rel(ys[0], OU.pack2(O.ac2_prime(X, W1, W2, Lm, Rm), Vl, Vr, list(QP), list(QP))) < 1e-13


def test_u1_pack_roundtrip():
    Ws, qw, mps, legs, Lm, Rm = _bond(12, 6, 40, 6, 2)
    Vl, Vr = legs[5], legs[7]
    X = np.tensordot(mps[5], mps[6], axes=([2], [0]))
    xp = u1_pack2(DT.from_numpy(X), sp(Vl), sp(Vr), QP, QP)
    assert np.array_equal(xp.numpy(), OU.pack2(X, Vl, Vr, list(QP), list(QP)))
    Xb = u1_unpack2(xp, sp(Vl), sp(Vr), QP, QP).numpy()
    assert np.array_equal(Xb, X)


@pytest.mark.parametrize("L,N,D,site", [(8, 4, 6, 4), (12, 6, 40, 6), (20, 10, 150, 9)])
def test_u1_twosite_and_envs(L, N, D, site):
    Ws, qw, mps, legs, Lm, Rm = _bond(L, N, D, site, 3 * L + D)
    Vl, Vm, Vr = legs[site - 1], legs[site], legs[site + 1]
    A, B = mps[site - 1], mps[site]
    x = fm.u1_twosite(DT.from_numpy(A), DT.from_numpy(B), sp(Vl), sp(Vm), sp(Vr), QP, QP)
    ref = OU.pack2(np.tensordot(A, B, axes=([2], [0])), Vl, Vr, list(QP), list(QP))
    assert rel(x.numpy(), ref) < 1e-14
    # updateleft over site `site` (legs Vl -> Vm), both kets different tensors
    rng = np.random.default_rng(L)
    Bk = A + 0.5 * rng.standard_normal(A.shape) * OU.allowed3(Vl, Vm, list(QP))
    W = Ws[site - 1]
    refL = O.updateleft(Lm, A, W, Bk)
    gL = fm.u1_updateleft(DT.from_numpy(Lm), DT.from_numpy(A), W, DT.from_numpy(Bk), sp(Vl),
                          sp(Vm), QP, qw[site - 1], qw[site]).numpy()
    assert rel(gL, refL) < 1e-13
    assert np.all(gL[~OU.allowed_env(Vm, qw[site])] == 0.0)
    # updateright over site `site + 1` (legs Vm -> Vr)
    W = Ws[site]
    Bk = B + 0.5 * rng.standard_normal(B.shape) * OU.allowed3(Vm, Vr, list(QP))
    refR = O.updateright(Rm, B, W, Bk)
    gR = fm.u1_updateright(DT.from_numpy(Rm), DT.from_numpy(B), W, DT.from_numpy(Bk), sp(Vm),
                           sp(Vr), QP, qw[site], qw[site + 1]).numpy()
    assert rel(gR, refR) < 1e-13
    assert np.all(gR[~OU.allowed_env(Vm, qw[site])] == 0.0)


@pytest.mark.parametrize("method", ["gesvd", "dm"])
@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("maxD,eps", [(100000, 0.0), (17, 0.0), (40, 1e-3)])
def test_u1_split(side, maxD, eps, method):
    Ws, qw, mps, legs, Lm, Rm = _bond(14, 7, 48, 7, 11)
    Vl, Vr = legs[6], legs[8]
    X = np.tensordot(mps[6], mps[7], axes=([2], [0]))
    tr = O.MPSTruncation(maxD, eps)
    xp = DT.from_numpy(OU.pack2(X, Vl, Vr, list(QP), list(QP)))
    A, S, B, Vm, err = fm.u1_split(xp, sp(Vl), sp(Vr), QP, QP, fm.MPSTruncation(maxD, eps), side,
                                   method)
    Ao, So, Bo, Vmo, erro = OU.u1_split(X, Vl, Vr, list(QP), list(QP), tr, side)
    # the density-matrix form resolves sigma to ~1e-8 sigma_max (squared in the Gram matrix)
    tol = 1e-12 if method == "gesvd" else 1e-9
    An, Bn = A.numpy(), B.numpy()
    if method == "dm" and eps == 0.0 and maxD > Vl.dim * 2:
        # x = A.B has rank-deficient sectors: the SVD keeps its ~1e-16 singular
        # values, the density-matrix form drops exact zeros; both reproduce x
        prod = np.tensordot(An, Bn, axes=([2], [0]))
        assert rel(prod, X / np.linalg.norm(X)) < tol
        return
    assert Vm.charges == tuple(Vmo.charges) and Vm.dims == tuple(Vmo.dims)
    assert np.abs(S.numpy() - So).max() < tol
    assert abs(err - erro) <= max(1e-10 * erro, tol * np.linalg.norm(X))
    prod = np.tensordot(An, Bn, axes=([2], [0]))
    assert rel(prod, np.tensordot(Ao, Bo, axes=([2], [0]))) < tol
    k = Vm.dim
    if side == 0:
        G = An.reshape(-1, k, order="F")
        assert np.abs(G.T @ G - np.eye(k)).max() < 1e-12
    else:
        G = Bn.reshape(k, -1, order="F")
        assert np.abs(G @ G.T - np.eye(k)).max() < 1e-12
    assert np.all(An[~OU.allowed3(Vl, Vmo, list(QP))] == 0.0)
    assert np.all(Bn[~OU.allowed3(Vmo, Vr, list(QP))] == 0.0)


def _states(L, N, D, seed):
    mps, legs = OU.random_u1_state(L, N, D, list(QP), np.random.default_rng(seed))
    psi = U1FiniteMPS([DT.from_numpy(A) for A in mps], [sp(l) for l in legs], QP)
    return mps, legs, psi


def test_u1_lanczos_matches_oracle():
    L, N = 10, 5
    Ws = heisenberg_xxz_mpo().site_tensors(L)
    mps, legs, psi = _states(L, N, 16, 4)
    env_o = OU.U1OracleEnv(Ws, mps, legs, list(QP), schur=True)
    env_o.right_canonicalize()
    u1_right_canonicalize_(psi, "gesvd")
    for i in range(1, L + 1):
        assert rel(psi[i].numpy(), env_o.mps[i - 1]) < 1e-11 or \
            rel(np.abs(psi[i].numpy()), np.abs(env_o.mps[i - 1])) < 1e-11
    m = fm.U1ExpectationCache(heisenberg_xxz_mpo(), psi)
    site = 1
    Vl, Vm, Vr = psi.spaces[1], psi.spaces[2], psi.spaces[3]
    x2 = fm.u1_twosite(psi[1], psi[2], Vl, Vm, Vr, QP, QP)
    op = fm.U1HeffOp(m.hstorage[1], m.hstorage[3], m.mpo[1], m.mpo[2], Vl, Vr, QP, QP,
                     m.qw[1], m.qw[2], m.qw[3])
    E, vec, info, k = op.lanczos(x2, 30, 1e-12)
    W1, W2 = Ws[0], Ws[1]
    Lh, Rh = env_o.hstorage[0], env_o.hstorage[2]
    X = np.tensordot(env_o.mps[0], env_o.mps[1], axes=([2], [0]))

    def f(v):
        return O.ac2_prime(v.reshape(X.shape, order="F"), W1, W2, Lh, Rh).ravel(order="F")

    Eo, vo, _, ko = O.simple_lanczos_solver(f, X.ravel(order="F"), 30, 1e-12)
    assert abs(E - Eo) < 1e-10 * abs(Eo)
    assert k == ko


@pytest.mark.parametrize("kmax", [3, 30])
def test_u1_lanczos_graph_equals_host_loop(kmax):
    """The graph-captured solve runs the same kernels in the same order as the
    host-driven loop: identical results, including early convergence (on a
    4-site chain the two-site space has a few states, so kmax 30 exhausts the
    Krylov space before kmax)."""
    L, N = 4, 2
    mps, legs, psi = _states(L, N, 8, 21)
    u1_right_canonicalize_(psi)
    m = fm.U1ExpectationCache(heisenberg_xxz_mpo(), psi)
    Vl, Vm, Vr = psi.spaces[2], psi.spaces[3], psi.spaces[4]
    x2 = fm.u1_twosite(psi[2], psi[3], Vl, Vm, Vr, QP, QP)
    op = fm.U1HeffOp(m.hstorage[2], m.hstorage[4], m.mpo[2], m.mpo[3], Vl, Vr, QP, QP,
                     m.qw[2], m.qw[3], m.qw[4])
    assert op.n < 30
    h = psi.handle
    g0 = h.graph_count()
    h.set_graphs(True)
    E1, v1, i1, k1 = op.lanczos(x2, kmax, 1e-12)
    assert h.graph_count() == g0 + 1
    E1b, v1b, _, _ = op.lanczos(x2, kmax, 1e-12)      # reused executable graph
    assert h.graph_count() == g0 + 2
    h.set_graphs(False)
    E2, v2, i2, k2 = op.lanczos(x2, kmax, 1e-12)
    h.set_graphs(True)
    assert (E1, i1, k1) == (E2, i2, k2) and E1b == E1
    assert np.array_equal(v1.numpy(), v2.numpy()) and np.array_equal(v1b.numpy(), v1.numpy())
    if kmax == 30:
        assert i1 == 0 and k1 < 30


def test_u1_projected_lanczos_graph_equals_host_loop():
    """fmpt_op_set_projectors on a block-sparse operator: the projection runs
    inside the captured graph (gated by the stop flag) and in the host-driven
    loop with identical results; the projected operator is _project!(H x), and
    projecting out the lowest eigenvector leaves the second eigenvalue."""
    L, N = 4, 2
    mps, legs, psi = _states(L, N, 8, 21)
    u1_right_canonicalize_(psi)
    m = fm.U1ExpectationCache(heisenberg_xxz_mpo(), psi)
    Vl, Vm, Vr = psi.spaces[2], psi.spaces[3], psi.spaces[4]
    x2 = fm.u1_twosite(psi[2], psi[3], Vl, Vm, Vr, QP, QP)
    op = fm.U1HeffOp(m.hstorage[2], m.hstorage[4], m.mpo[2], m.mpo[3], Vl, Vr, QP, QP,
                     m.qw[2], m.qw[3], m.qw[4])
    n = op.n
    H = np.empty((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        H[:, j] = op(DT.from_numpy(e)).numpy()
    assert np.abs(H - H.T).max() < 1e-12
    w, V = np.linalg.eigh(H)
    p0 = DT.from_numpy(V[:, 0])
    op.set_projectors([p0])
    xr = np.random.default_rng(3).standard_normal(n)
    y = op(DT.from_numpy(xr)).numpy()
    Hx = H @ xr
    assert np.abs(y - (Hx - np.dot(Hx, V[:, 0]) * V[:, 0])).max() < 1e-12 * np.abs(Hx).max()
    x0 = x2.copy()
    fm.project_(x0, [p0])
    h = psi.handle
    h.set_graphs(True)
    g0 = h.graph_count()
    E1, v1, i1, k1 = op.lanczos(x0, 30, 1e-12)
    assert h.graph_count() == g0 + 1
    h.set_graphs(False)
    E2, v2, i2, k2 = op.lanczos(x0, 30, 1e-12)
    h.set_graphs(True)
    assert (E1, i1, k1) == (E2, i2, k2)
    assert np.array_equal(v1.numpy(), v2.numpy())
    assert abs(E1 - w[1]) < 1e-10


@pytest.mark.parametrize("L,N,D,model", [(12, 6, 48, "xxz"), (12, 4, 48, "xxz"),
                                         (10, 5, 40, "j1j2")])
def test_u1_dmrg2_vs_ed_and_oracle(L, N, D, model):
    mpo = heisenberg_xxz_mpo() if model == "xxz" else j1j2_heisenberg_mpo(1.0, 0.5)
    Ws = mpo.site_tensors(L)
    mps, legs, psi = _states(L, N, 8, 7)
    env_o = OU.U1OracleEnv(Ws, mps, legs, list(QP), schur=True)
    env_o.right_canonicalize()
    u1_right_canonicalize_(psi)
    alg = fm.DMRG2(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(D, 1e-12), verbosity=0)
    m = fm.U1ExpectationCache(mpo, psi)
    tr = O.MPSTruncation(D, 1e-12)
    for sweep in range(3):
        Eg, dg = fm.sweep_(m, alg)
        Eo, do = OU.u1_dmrg2_sweep(env_o, tr, 30, 1e-12)
        assert np.abs(np.asarray(Eg) - np.asarray(Eo)).max() < 1e-9 * abs(Eo[-1])
    if model == "xxz":
        e_ed = xxz_ground_energy(L, nup=N)
    else:
        from oracle.ed import j1j2_ground_energy
        e_ed = j1j2_ground_energy(L, 1.0, 0.5, nup=N)
    assert abs(Eg[-1] - e_ed) < 1e-10 * abs(e_ed)
    assert abs(fm.expectation(psi, mpo) - Eg[-1]) < 1e-10 * abs(e_ed)
    assert psi.total_charge == N


def test_u1_dmrg2_density_matrix_split():
    """svd="dm" (batched density-matrix split) converges to the same energy."""
    L, N = 12, 6
    mpo = heisenberg_xxz_mpo()
    mps, legs, psi = _states(L, N, 8, 12)
    u1_right_canonicalize_(psi)
    alg = fm.DMRG2(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(64, 1e-12), verbosity=0,
                   svd="dm")
    m = fm.U1ExpectationCache(mpo, psi)
    for _ in range(3):
        E, _ = fm.sweep_(m, alg)
    assert abs(E[-1] - xxz_ground_energy(L, nup=N)) < 1e-10 * abs(E[-1])


def test_u1_dmrg2_matches_dense_path():
    """Same chain, dense FP64 path vs U(1) path: same ground energy."""
    L, N = 12, 6
    mpo = heisenberg_xxz_mpo()
    mps, legs, psi = _states(L, N, 8, 9)
    u1_right_canonicalize_(psi)
    dense = fm.FiniteMPS([DT.from_numpy(A.numpy()) for A in psi.data])
    alg = fm.DMRG2(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(64, 1e-12), verbosity=0)
    m1 = fm.U1ExpectationCache(mpo, psi)
    m2 = fm.environments(mpo, dense)
    for _ in range(3):
        E1, _ = fm.sweep_(m1, alg)
        E2, _ = fm.sweep_(m2, alg)
    assert abs(E1[-1] - E2[-1]) < 1e-10 * abs(E2[-1])
    assert abs(E1[-1] - xxz_ground_energy(L, nup=N)) < 1e-10 * abs(E1[-1])


def test_u1_rejects_bad_input():
    Ws, qw, mps, legs, Lm, Rm = _bond(8, 4, 6, 4, 1)
    Vl, Vr = legs[3], legs[5]
    dL, dR = DT.from_numpy(Lm), DT.from_numpy(Rm)
    bad = Ws[3].copy()
    bad[0, 0, 1, 0] = 1.0        # S+ channel on a charge-diagonal entry
    with pytest.raises(fm.FMPTError):
        fm.U1HeffOp(dL, dR, bad, Ws[4], sp(Vl), sp(Vr), QP, QP, qw[3], qw[4], qw[5])
    with pytest.raises(fm.FMPTError):   # wrong channel charges
        fm.U1HeffOp(dL, dR, Ws[3], Ws[4], sp(Vl), sp(Vr), QP, QP, qw[3], [0, 0, 0, 0, 0], qw[5])


def test_grouped_barrier_timeout_is_reported_and_context_survives():
    """Failure detection without a GPU fault: the grouped launch's grid barrier is made to
    wait for an arrival that never comes (fmpt_set_wait_test hold), gives up after its
    0.2 s bound, sets the status word and returns; fmpt_synchronize reports
    FMPT_ERR_TIMEOUT, and after the hook is cleared the same operator gives the right
    result again on the same context."""
    from finitemptools_gb300._native import FMPTError
    L, N, D, site = 10, 5, 20, 5
    Ws, qw, mps, legs, Lm, Rm = _bond(L, N, D, site, 77)
    Vl, Vr = legs[site - 1], legs[site + 1]
    W1, W2 = Ws[site - 1], Ws[site]
    X = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
    ref = OU.pack2(O.ac2_prime(X, W1, W2, Lm, Rm), Vl, Vr, list(QP), list(QP))
    h = fm.default_handle()
    dL, dR = DT.from_numpy(Lm), DT.from_numpy(Rm)
    op = fm.U1HeffOp(dL, dR, W1, W2, sp(Vl), sp(Vr), QP, QP, qw[site - 1], qw[site],
                     qw[site + 1])
    x = DT.from_numpy(OU.pack2(X, Vl, Vr, list(QP), list(QP)))
    assert rel(op(x).numpy(), ref) < 1e-13          # built, tuned and correct
    h.set_wait_test(0.2, hold=True)
    try:
        op(x)
        with pytest.raises(FMPTError) as ei:
            h.synchronize()
        assert ei.value.status == -5
    finally:
        h.set_wait_test(0.0, hold=False)
    h.synchronize()                                  # the status word was cleared
    assert rel(op(x).numpy(), ref) < 1e-13
