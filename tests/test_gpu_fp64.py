"""Parity of the plain FP64 device path against the CPU oracle.

Bar: H_eff*x within 1e-12 relative (Frobenius) of the oracle; sweep energies
within 1e-10.  Environment updates, SVD, QR/LQ and
the Krylov solvers are checked at the same level.  Shapes include odd and
tiny bond dimensions (1, 3, 7, 33) so every tile edge of the kernels runs.
"""

import json
import os

import numpy as np
import pytest

import oracle as O
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300.utilities import FiniteMPO, heisenberg_xxz_mpo, j1j2_heisenberg_mpo, tfi_mpo

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def rnd(rng, shape, cplx):
    a = rng.standard_normal(shape)
    if cplx:
        a = a + 1j * rng.standard_normal(shape)
    return a


def herm_env(rng, D, w, cplx):
    E = rnd(rng, (D, w, D), cplx)
    return 0.5 * (E + np.conj(np.transpose(E, (2, 1, 0))))


def rand_mpo(rng, wl, d, wr, cplx, density=0.5):
    W = rnd(rng, (wl, d, wr, d), cplx)
    mask = rng.random((wl, 1, wr, 1)) < density
    return W * mask


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("Dl,Dr,w", [(1, 3, 5), (7, 5, 5), (16, 16, 5), (33, 20, 8)])
def test_ac2_prime_fp64(cplx, Dl, Dr, w):
    rng = np.random.default_rng(Dl * 100 + Dr + cplx)
    W1 = heisenberg_xxz_mpo(1.0, 0.7, 0.3)[1].dense() if w == 5 else rand_mpo(rng, w, 2, w, cplx)
    W2 = rand_mpo(rng, w, 2, w, cplx) if cplx else W1
    x = rnd(rng, (Dl, 2, 2, Dr), cplx)
    L = herm_env(rng, Dl, w, cplx)
    R = herm_env(rng, Dr, w, cplx)
    ref = O.ac2_prime(x, W1, W2, L, R)
    y = fm.ac2_prime(DT.from_numpy(x), W1, W2, DT.from_numpy(L), DT.from_numpy(R)).numpy()
    assert rel(y, ref) < 1e-12


def test_ac2_prime_golden_fixture():
    g = np.load(os.path.join(GOLDEN, "ac2_D12.npz"))
    y = fm.ac2_prime(DT.from_numpy(g["x"]), g["W"], g["W"], DT.from_numpy(g["L"]),
                     DT.from_numpy(g["R"])).numpy()
    assert rel(y, g["y"]) < 1e-12


def test_ac2_prime_boundary_mpo_shapes():
    """FiniteMPO(h, L) cuts the grid at the chain ends: wl=1 on the left."""
    rng = np.random.default_rng(5)
    h = heisenberg_xxz_mpo(1.0, 1.0, 0.2)
    Ws = FiniteMPO(h, 4)
    x = rng.standard_normal((1, 2, 2, 4))
    L = np.ones((1, 1, 1))
    R = herm_env(rng, 4, 5, False)
    ref = O.ac2_prime(x, Ws[0], Ws[1], L, R)
    y = fm.ac2_prime(DT.from_numpy(x), Ws[0], Ws[1], DT.from_numpy(L), DT.from_numpy(R)).numpy()
    assert rel(y, ref) < 1e-12


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("Dl,Dr,w,d", [(1, 2, 3, 2), (9, 13, 3, 2), (24, 24, 8, 2), (6, 6, 4, 4)])
def test_ac_prime_and_c_prime_fp64(cplx, Dl, Dr, w, d):
    rng = np.random.default_rng(Dl + 7 * Dr + cplx)
    W = rand_mpo(rng, w, d, w, cplx)
    x = rnd(rng, (Dl, d, Dr), cplx)
    L = herm_env(rng, Dl, w, cplx)
    R = herm_env(rng, Dr, w, cplx)
    y = fm.ac_prime(DT.from_numpy(x), W, DT.from_numpy(L), DT.from_numpy(R)).numpy()
    assert rel(y, O.ac_prime(x, W, L, R)) < 1e-12
    C = rnd(rng, (Dl, Dr), cplx)
    yc = fm.c_prime(DT.from_numpy(C), DT.from_numpy(L), DT.from_numpy(R)).numpy()
    assert rel(yc, O.c_prime(C, L, R)) < 1e-12


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("Dl,Dr,wl,wr,d", [(1, 2, 1, 5, 2), (5, 10, 5, 5, 2), (17, 31, 8, 8, 2),
                                           (12, 12, 3, 1, 3)])
def test_env_updates_fp64(cplx, Dl, Dr, wl, wr, d):
    rng = np.random.default_rng(Dl * 3 + Dr + 11 * cplx)
    W = rand_mpo(rng, wl, d, wr, cplx, density=0.7)
    A = rnd(rng, (Dl, d, Dr), cplx)
    B = rnd(rng, (Dl, d, Dr), cplx)
    Lh = rnd(rng, (Dl, wl, Dl), cplx)
    Rh = rnd(rng, (Dr, wr, Dr), cplx)
    gl = fm.updateleft(DT.from_numpy(Lh), DT.from_numpy(A), W, DT.from_numpy(B)).numpy()
    assert rel(gl, O.updateleft(Lh, A, W, B)) < 1e-12
    gr = fm.updateright(DT.from_numpy(Rh), DT.from_numpy(A), W, DT.from_numpy(B)).numpy()
    assert rel(gr, O.updateright(Rh, A, W, B)) < 1e-12
    # operator-less overlap updates (mpo/transfer.jl:37-45)
    Lo = rnd(rng, (Dl, 2, Dl), cplx)
    go = fm.updateleft(DT.from_numpy(Lo), DT.from_numpy(A), None, DT.from_numpy(B)).numpy()
    assert rel(go, O.updateleft_overlap(Lo, A, B)) < 1e-12
    Ro = rnd(rng, (Dr, 2, Dr), cplx)
    go = fm.updateright(DT.from_numpy(Ro), DT.from_numpy(A), None, DT.from_numpy(B)).numpy()
    assert rel(go, O.updateright_overlap(Ro, A, B)) < 1e-12


@pytest.mark.parametrize("kmax", [1, 5, 30])
@pytest.mark.parametrize("reorth", [False, True])
def test_lanczos_matches_restatement(kmax, reorth):
    from helpers import xz_mpo, sym_env
    rng = np.random.default_rng(kmax)
    D = 10
    W = xz_mpo()
    L = sym_env(rng, D, 4)
    R = sym_env(rng, D, 4)
    x = rng.standard_normal((D, 2, 2, D))
    E0, v0, info0, k0 = O.simple_lanczos_solver(
        lambda v: O.ac2_prime(v.reshape(x.shape, order="F"), W, W, L, R).ravel(order="F"),
        x.ravel(order="F"), kmax, 1e-12)
    op = fm.HeffOp("ac2", DT.from_numpy(L), DT.from_numpy(R), W1=W, W2=W)
    E1, v1, info1, k1 = op.lanczos(DT.from_numpy(x), kmax, 1e-12, reorth=reorth)
    assert k1 == k0 and info1 == info0
    v1 = v1.numpy().ravel(order="F")
    if not reorth:   # the reference's recurrence, step for step
        assert abs(E1 - E0) <= 1e-12 * max(1.0, abs(E0))
        s = np.sign(np.vdot(v0, v1))
        assert np.linalg.norm(v1 * s - v0) < 1e-9
    # either way: a Ritz pair of the symmetric H_eff, never below its spectrum
    H = np.array([O.ac2_prime(e.reshape(x.shape, order="F"), W, W, L, R).ravel(order="F")
                  for e in np.eye(x.size)]).T
    lam = np.linalg.eigvalsh(H)
    assert E1 >= lam[0] - 1e-9 * abs(lam[0])
    rq = v1 @ H @ v1 / (v1 @ v1)
    assert abs(rq - E1) < 1e-6 * abs(E1)


def test_lanczos_early_exit():
    """beta < btol after the first step (simple_lanczos.jl:86-89)."""
    D = 4
    W = np.zeros((1, 2, 1, 2)); W[0, :, 0, :] = np.diag([1.0, 2.0])
    L = np.eye(D).reshape(D, 1, D)
    R = np.eye(D).reshape(D, 1, D)
    x = np.zeros((D, 2, 2, D)); x[:, 0, 0, :] = np.eye(D)
    op = fm.HeffOp("ac2", DT.from_numpy(L), DT.from_numpy(R), W1=W, W2=W)
    E, v, info, k = op.lanczos(DT.from_numpy(x), 10, 1e-12)
    # x lives in the s1=s2=0 eigenspace of W1 (x) W2 = diag(1,2) (x) diag(1,2): E = 1
    assert k == 1 and abs(E - 1.0) < 1e-14


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n", [(40, 12), (12, 40), (64, 64), (1, 7)])
def test_svd_trunc_qr_lq(cplx, m, n):
    rng = np.random.default_rng(m * n + cplx)
    M = rnd(rng, (m, n), cplx)
    # graded spectrum so that the cutoff bites
    U0, s0, V0 = np.linalg.svd(M, full_matrices=False)
    s0 = np.logspace(0, -14, len(s0))
    M = (U0 * s0) @ V0
    tr = fm.MPSTruncation(max(1, min(m, n) - 2), 1e-10)
    U, S, Vt, err = fm.stable_tsvd(DT.from_numpy(M), m, n, tr)
    k_ref, err_ref = O.mps_truncate(s0, O.MPSTruncation(tr.D, tr.eps))
    assert S.shape[0] == k_ref
    assert abs(err - err_ref) < 1e-12
    s = S.numpy()
    assert np.allclose(s, s0[:k_ref], rtol=1e-12, atol=1e-15)
    Mk = (U.numpy() * s) @ Vt.numpy()
    Mref = (U0[:, :k_ref] * s0[:k_ref]) @ V0[:k_ref]
    assert rel(Mk, Mref) < 1e-11
    Q, R = fm.leftorth(DT.from_numpy(M), m, n)
    Qn, Rn = Q.numpy(), R.numpy()
    assert rel(Qn @ Rn, M) < 1e-13
    assert np.allclose(Qn.conj().T @ Qn, np.eye(Qn.shape[1]), atol=1e-13)
    assert np.allclose(np.tril(Rn, -1), 0)
    Lm, Q2 = fm.rightorth(DT.from_numpy(M), m, n)
    Ln, Q2n = Lm.numpy(), Q2.numpy()
    assert rel(Ln @ Q2n, M) < 1e-13
    assert np.allclose(Q2n @ Q2n.conj().T, np.eye(Q2n.shape[0]), atol=1e-13)


@pytest.mark.parametrize("m,n,cplx,zero_col", [(128, 64, True, None), (64, 128, True, None),
                                              (100, 100, False, None), (1, 5, True, None),
                                              (7, 1, False, None), (50, 20, True, 3),
                                              (300, 200, True, None), (256, 40, False, 39)])
def test_qr_conventions_match_lapack(m, n, cplx, zero_col):
    """leftorth (fmpt_qr, cuSOLVER geqrf/ungqr) against numpy's geqrf/ungqr factors, entry
    by entry: the same Householder conventions (real diagonal of R, beta = -sign(Re a)
    |(a, x)|) give the same Q and R up to rounding, so the gauge of the moves matches the
    reference's LAPACK QR; a zero column takes the tau = 0 reflector."""
    rng = np.random.default_rng(m * 7 + n)
    M = rnd(rng, (m, n), cplx)
    if zero_col is not None:
        M[:, zero_col] = 0.0
    Q, R = fm.leftorth(DT.from_numpy(M), m, n)
    Qn, Rn = Q.numpy(), R.numpy()
    Qr, Rr = np.linalg.qr(M)
    assert np.abs(Qn - Qr).max() < 1e-12 * max(1, m), np.abs(Qn - Qr).max()
    assert np.abs(Rn - Rr).max() < 1e-12 * np.abs(Rr).max() * max(1, m)
    assert np.allclose(np.imag(np.diag(Rn)), 0)
    Lm, Q2 = fm.rightorth(DT.from_numpy(M), m, n)
    assert rel(Lm.numpy() @ Q2.numpy(), M) < 1e-13


@pytest.mark.parametrize("m,n,cplx", [(128, 64, True), (128, 64, False), (96, 96, True),
                                       (512, 8, True), (33, 17, False), (200, 150, True),
                                       (3, 1, True)])
def test_cluster_qr_equals_cusolver(m, n, cplx):
    """The thread-block-cluster QR of small tall panels against cuSOLVER geqrf/ungqr on the
    same input, entry by entry (the same LAPACK reflector conventions; a zero column takes
    tau = 0 in both).  A rank-deficient panel (a repeated column) has no unique Q past its
    rank -- rounding noise picks those columns -- so there only Q R = M, the orthonormality
    of Q and the triangular R with real diagonal are checked."""
    rng = np.random.default_rng(m + 3 * n)
    M = rnd(rng, (m, n), cplx)
    if n >= 4:
        M[:, n - 1] = 0.0
    h = fm.default_handle()
    out = {}
    try:
        for on in (False, True):
            h.set_cluster_qr(on)
            Q, R = fm.leftorth(DT.from_numpy(M), m, n)
            Lm, Q2 = fm.rightorth(DT.from_numpy(M.conj().T.copy()), n, m)
            out[on] = (Q.numpy(), R.numpy(), Lm.numpy(), Q2.numpy())
    finally:
        h.set_cluster_qr(True)
    for a, b in zip(out[False], out[True]):
        assert np.abs(a - b).max() < 1e-12 * max(1, m) * max(1.0, np.abs(a).max())
    if n >= 4:
        M[:, 2] = M[:, 1]                     # rank deficient
    Q, R = fm.leftorth(DT.from_numpy(M), m, n)
    Qn, Rn = Q.numpy(), R.numpy()
    assert rel(Qn @ Rn, M) < 1e-13
    assert np.allclose(Qn.conj().T @ Qn, np.eye(n), atol=1e-13)
    assert np.allclose(np.tril(Rn, -1), 0) and np.allclose(np.imag(np.diag(Rn)), 0)


@pytest.mark.parametrize("cplx", [False, True])
def test_exponentiate_matches_exact(cplx):
    import scipy.linalg
    rng = np.random.default_rng(3)
    D, w, d = 6, 3, 2
    W = tfi_mpo([1.1] * 4)[2].dense()
    L = herm_env(rng, D, w, cplx)
    R = herm_env(rng, D, w, cplx)
    x = rnd(rng, (D, d, D), cplx)
    H = np.zeros((x.size, x.size), dtype=complex)
    for i in range(x.size):
        e = np.zeros(x.size); e[i] = 1
        H[:, i] = O.ac_prime(e.reshape(x.shape, order="F"), W, L, R).ravel(order="F")
    t = -0.3j if cplx else -0.2
    ref = scipy.linalg.expm(t * H) @ x.ravel(order="F")
    dt = np.complex128 if cplx else np.float64
    op = fm.HeffOp("ac", DT.from_numpy(L), DT.from_numpy(R), W1=W, dtype=dt)
    y = op.exponentiate(t, DT.from_numpy(x.astype(dt)), tol=1e-12, krylovdim=20).numpy()
    assert rel(y.ravel(order="F"), ref) < 1e-10


def _oracle_and_device_dmrg(mpo_dev, mpo_or, L, d, D0, sweeps, trunc, kmax, tol, seed,
                            schur=False):
    rng = np.random.default_rng(seed)
    st = O.randommps(L, d, D0, rng)
    st, _ = O.canonicalize(st, normalize=True)
    env_o = O.environments(mpo_or, st, schur=schur)
    env_d = fm.environments(mpo_dev, fm.FiniteMPS.from_numpy(st))
    alg = fm.DMRG2(eig_maxiter=kmax, eig_tol=tol, trunc=fm.MPSTruncation(trunc[0], trunc[1]))
    out = []
    for _ in range(sweeps):
        Eo, do = O.dmrg2_sweep(env_o, O.MPSTruncation(*trunc), kmax, tol)
        Ed, dd = fm.sweep_(env_d, alg)
        out.append((Eo, do, Ed, dd))
    return out, env_o, env_d


def test_dmrg2_sweep_parity_small():
    """Plain DMRG2 on a Schur MPOHamiltonian and on its FiniteMPO embedding:
    every Ritz value of every bond matches the oracle to 1e-10."""
    L = 10
    h = heisenberg_xxz_mpo(1.0, 1.0, 0.3)
    res, env_o, env_d = _oracle_and_device_dmrg(FiniteMPO(h, L), FiniteMPO(h, L), L, 2, 4, 3,
                                                (16, 1e-10), 20, 1e-12, 1)
    for Eo, do, Ed, dd in res:
        assert len(Eo) == len(Ed) == 2 * L - 3
        assert np.max(np.abs(np.array(Eo) - np.array(Ed))) < 1e-10
    res, _, _ = _oracle_and_device_dmrg(h, h.site_tensors(L), L, 2, 4, 2, (16, 1e-10), 20, 1e-12,
                                        2, schur=True)
    for Eo, do, Ed, dd in res:
        assert np.max(np.abs(np.array(Eo) - np.array(Ed))) < 1e-10
    # expectation(psi, h, psi) on the device equals the oracle's on the same state
    e_dev = fm.expectation(env_d.mps, FiniteMPO(h, L))
    e_or = O.expectation_mpo([A.numpy() for A in env_d.mps], FiniteMPO(h, L))
    assert abs(e_dev - e_or) < 1e-10


def test_dmrg2_config_xxz_L20_vs_ed_and_oracle():
    """XXZ L=20, Delta=1, D0=8 random right-canonical start, 4 sweeps of
    DMRG2(eig_maxiter=30, eig_tol=1e-12, MPSTruncation(64, 1e-10)):
    energies within 1e-10 of the oracle and the final energy at the exact
    diagonalisation value (2^20 states, committed fixture)."""
    L = 20
    h = heisenberg_xxz_mpo(1.0, 1.0, 0.0)
    res, _, _ = _oracle_and_device_dmrg(FiniteMPO(h, L), FiniteMPO(h, L), L, 2, 8, 4,
                                        (64, 1e-10), 30, 1e-12, 20)
    for Eo, do, Ed, dd in res:
        assert np.max(np.abs(np.array(Eo) - np.array(Ed))) < 1e-10
    with open(os.path.join(GOLDEN, "exact_energies.json")) as f:
        E_ed = json.load(f)["xxz_L20_J1_Jzz1_hz0"]
    assert abs(res[-1][2][-1] - E_ed) < 1e-6 * abs(E_ed)


def test_dmrg1_parity():
    L = 8
    h = heisenberg_xxz_mpo(1.0, 1.0, 0.2)
    rng = np.random.default_rng(4)
    st, _ = O.canonicalize(O.randommps(L, 2, 4, rng), normalize=True)
    env_o = O.environments(FiniteMPO(h, L), st)
    env_d = fm.environments(FiniteMPO(h, L), fm.FiniteMPS.from_numpy(st))
    alg = fm.DMRG1(D=8, eig_maxiter=20)
    for _ in range(3):
        Eo, do = O.dmrg1_sweep(env_o, D=8, eig_maxiter=20)
        Ed, dd = fm.sweep_(env_d, alg)
        assert np.max(np.abs(np.array(Eo) - np.array(Ed))) < 1e-10
        assert abs(do - dd) < 1e-8


def test_tdvp1_parity():
    """One-site TDVP, complex: <Z_i> after 3 steps agrees with the oracle."""
    L, D = 6, 8
    rng = np.random.default_rng(12)
    hs = 1.0 + 0.1 * rng.standard_normal(L)
    h = tfi_mpo(hs)
    st = O.randommps(L, 2, D, rng, dtype=np.complex128)
    st, _ = O.canonicalize(st, normalize=True)
    mpo = [W.astype(complex) for W in FiniteMPO(h, L)]
    env_o = O.environments(mpo, st)
    env_d = fm.environments(FiniteMPO(h, L), fm.FiniteMPS.from_numpy(st, dtype=np.complex128))
    alg = fm.TDVP1(stepsize=-0.05j, D=D, exptol=1e-10, krylovdim=20)
    Z = np.diag([-1.0, 1.0])
    for _ in range(3):
        O.tdvp1_sweep(env_o, -0.05j, D=D, exptol=1e-10, krylovdim=20)
        fm.sweep_(env_d, alg)
    zo = [O.single_site_expectation(env_o.mps, i, Z).real for i in range(1, L + 1)]
    zd = [fm.expectation_local(env_d.mps, i, Z).real for i in range(1, L + 1)]
    assert np.max(np.abs(np.array(zo) - np.array(zd))) < 1e-8


def test_launch_counter_moves():
    h = fm.default_handle()
    n0 = h.launch_count()
    x = DT.from_numpy(np.ones((3, 2, 2, 3)))
    W = heisenberg_xxz_mpo()[1].dense()
    E = DT.from_numpy(np.ones((3, 5, 3)))
    fm.ac2_prime(x, W, W, E, E)
    assert h.launch_count() >= n0 + 3


def test_bad_shapes_raise():
    x = DT.from_numpy(np.ones((3, 2, 2, 4)))
    W = heisenberg_xxz_mpo()[1].dense()
    E = DT.from_numpy(np.ones((3, 5, 3)))
    with pytest.raises(ValueError):
        fm.ac2_prime(x, W, W, E, E)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n,side", [(40, 24, 0), (40, 24, 1), (24, 40, 0), (64, 64, 1)])
def test_dm_split(cplx, m, n, side):
    """Density-matrix split: the isometric factor is exactly isometric and
    the product is the rank-k truncation of M (singular values >= 1e-6)."""
    from finitemptools_gb300.auxiliary import dm_split
    rng = np.random.default_rng(m + n + side)
    U0, _ = np.linalg.qr(rnd(rng, (m, m), cplx))
    V0, _ = np.linalg.qr(rnd(rng, (n, n), cplx))
    r = min(m, n)
    s0 = np.logspace(0, -6, r)
    M = (U0[:, :r] * s0) @ V0[:, :r].conj().T
    k_max = r - 3
    A, S, B, err = dm_split(DT.from_numpy(M), m, n, fm.MPSTruncation(k_max, 1e-9), side)
    An, Sn, Bn = A.numpy(), S.numpy(), B.numpy()
    assert Sn.shape[0] == k_max
    assert np.allclose(Sn, s0[:k_max], rtol=1e-8)
    if side == 0:
        assert np.allclose(An.conj().T @ An, np.eye(k_max), atol=1e-13)
    else:
        assert np.allclose(Bn @ Bn.conj().T, np.eye(k_max), atol=1e-13)
    Mk = (U0[:, :k_max] * s0[:k_max]) @ V0[:, :k_max].conj().T
    assert rel(An @ Bn, Mk) < 1e-10
    assert abs(err - np.linalg.norm(s0[k_max:])) < 1e-10


@pytest.mark.parametrize("prec,cplx", [("fp64", True), ("fp64", False), ("tf32x3", True)])
def test_exponentiate_graph_equals_direct(prec, cplx):
    """The graph-captured Arnoldi basis (one CUDA graph per operator structure, updated in
    place across operators) gives bit-identical exponentials to the direct launches."""
    rng = np.random.default_rng(9)
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    dt = np.complex128 if cplx else np.float64
    h = fm.default_handle()

    def case(seed):
        r = np.random.default_rng(seed)
        L = r.standard_normal((24, 5, 24))
        R = r.standard_normal((20, 5, 20))
        L, R = 0.5 * (L + L.transpose(2, 1, 0)), 0.5 * (R + R.transpose(2, 1, 0))
        x = r.standard_normal((24, 2, 20))
        return (DT.from_numpy(L, dtype=dt), DT.from_numpy(R, dtype=dt),
                DT.from_numpy(x, dtype=dt))

    t = -0.05j if cplx else -0.05
    outs = {}
    for graphs in (False, True):
        h.set_graphs(graphs)
        res = []
        for seed in (1, 2, 1):        # fresh, updated in place, updated back
            L, R, x = case(seed)
            op = fm.HeffOp("ac", L, R, W1=W, precision=prec, dtype=dt)
            res.append(op.exponentiate(t, x, 1e-10, 20).numpy())
            res.append(op.exponentiate(t, x, 1e-10, 20).numpy())
        outs[graphs] = res
    h.set_graphs(True)
    for a, b in zip(outs[False], outs[True]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("graphs", [False, True])
@pytest.mark.parametrize("prec,cplx", [("fp64", True), ("fp64", False), ("tf32x3", True)])
def test_fused_krylov_step_equals_separate_launches(prec, cplx, graphs):
    """The fused orthogonalisation step (one cooperative launch per Arnoldi vector) gives
    bit-identical exponentials and quadrature-node vectors to the seven separate launches,
    with and without graph capture, and the Krylov exponential stays within 1e-10 of the
    dense matrix exponential."""
    import scipy.linalg
    from finitemptools_gb300 import adjoint as AD
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.2)[1].dense()
    dt = np.complex128 if cplx else np.float64
    h = fm.default_handle()
    r = np.random.default_rng(31)
    Ln = r.standard_normal((24, 5, 24))
    Rn = r.standard_normal((20, 5, 20))
    Ln, Rn = 0.5 * (Ln + Ln.transpose(2, 1, 0)), 0.5 * (Rn + Rn.transpose(2, 1, 0))
    xn = r.standard_normal((24, 2, 20))
    L, R, x = (DT.from_numpy(a, dtype=dt) for a in (Ln, Rn, xn))
    t = -0.05j if cplx else -0.05
    h.set_graphs(graphs)
    outs = {}
    try:
        for fused in (False, True):
            h.set_fused_krylov(fused)
            op = fm.HeffOp("ac", L, R, W1=W, precision=prec, dtype=dt)
            y1 = op.exponentiate(t, x, 1e-10, 20).numpy()
            y2 = op.exponentiate(t, x, 1e-10, 20).numpy()
            vs, err = AD.expm_nodes(op, t, x, np.array([0.25, 1.0]), 20)
            outs[fused] = [y1, y2] + [v.numpy() for v in vs]
    finally:
        h.set_fused_krylov(True)
        h.set_graphs(True)
    for a, b in zip(outs[False], outs[True]):
        assert np.array_equal(a, b)
    if prec == "fp64":
        from oracle import tdvp_adjoint as TA
        Hd = TA._heff("ac", W, Ln, Rn, xn.shape)
        ref = scipy.linalg.expm(t * Hd) @ xn.ravel(order="F")
        assert rel(outs[True][0].ravel(order="F"), ref) < 1e-10


def test_fused_krylov_barrier_timeout_is_reported_and_context_survives():
    """Failure detection without a GPU fault on the fused Krylov step: its grid barriers
    are made to wait for an arrival that never comes (fmpt_set_wait_test hold), give up
    after the 0.2 s bound, set the status word and return; the exponential reports
    FMPT_ERR_TIMEOUT, and with the hook cleared the same operator gives the same result
    as before on the same context."""
    from finitemptools_gb300._native import FMPTError
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    h = fm.default_handle()
    r = np.random.default_rng(32)
    Ln = r.standard_normal((16, 5, 16))
    Rn = r.standard_normal((16, 5, 16))
    Ln, Rn = 0.5 * (Ln + Ln.transpose(2, 1, 0)), 0.5 * (Rn + Rn.transpose(2, 1, 0))
    L, R = DT.from_numpy(Ln, dtype=np.complex128), DT.from_numpy(Rn, dtype=np.complex128)
    x = DT.from_numpy(r.standard_normal((16, 2, 16)), dtype=np.complex128)
    op = fm.HeffOp("ac", L, R, W1=W, dtype=np.complex128)
    ref = op.exponentiate(-0.05j, x, 1e-10, 10).numpy()
    h.set_wait_test(0.2, hold=True)
    try:
        with pytest.raises(FMPTError) as ei:
            op.exponentiate(-0.05j, x, 1e-10, 10)
            h.synchronize()
        assert ei.value.status == -5
    finally:
        h.set_wait_test(0.0, hold=False)
    h.synchronize()
    assert np.array_equal(op.exponentiate(-0.05j, x, 1e-10, 10).numpy(), ref)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("m,n,eps", [(300, 256, 1e-10), (256, 384, 1e-9)])
def test_dm_split_resolves_graded_spectrum(cplx, side, m, n, eps):
    """A spectrum logspace(0, -12): squaring resolves sigma only to ~1e-7 sigma_max, so the
    split refines its tail (rotations by the eigenvectors of the tail rows' Gram matrix,
    after projecting out the resolved rows).  The kept count equals the MPSTruncation rule
    (truncation.jl:27-47) on the exact singular values, the kept sigma match them to 1e-7
    relative (1e-8 above 1e-4 sigma_max), and the product is the rank-k truncation of M."""
    from finitemptools_gb300.auxiliary import dm_split
    rng = np.random.default_rng(m + n + 10 * side + cplx)
    r = min(m, n)
    U0, _ = np.linalg.qr(rnd(rng, (m, r), cplx))
    V0, _ = np.linalg.qr(rnd(rng, (n, r), cplx))
    s0 = np.logspace(0, -12, r)
    M = (U0 * s0) @ V0.conj().T
    tr = fm.MPSTruncation(r, eps)
    k_ref, err_ref = O.mps_truncate(s0, tr)
    A, S, B, err = dm_split(DT.from_numpy(M), m, n, tr, side)
    An, Sn, Bn = A.numpy(), S.numpy(), B.numpy()
    assert Sn.shape[0] == k_ref
    relerr = np.abs(Sn / s0[:k_ref] - 1.0)
    assert relerr.max() < 1e-7, relerr.max()
    assert relerr[s0[:k_ref] > 1e-4].max() < 1e-8
    if side == 0:
        assert np.allclose(An.conj().T @ An, np.eye(k_ref), atol=1e-12)
    else:
        assert np.allclose(Bn @ Bn.conj().T, np.eye(k_ref), atol=1e-12)
    Mk = (U0[:, :k_ref] * s0[:k_ref]) @ V0[:, :k_ref].conj().T
    assert rel(An @ Bn, Mk) < 1e-10
    assert abs(err - err_ref) < 1e-12
