"""Mixed-precision (tcgen05) contractions against the FP64 oracle.

Each precision form states its error bound against FP64 (relative Frobenius
norm of H_eff*x), the bounds of the mixed-precision H_eff*x workload:
  3xTF32 (hi/lo split, FP32 accumulation)  < 2e-6
  TF32   (FP32 accumulation)               < 3e-3
  BF16   (FP32 accumulation)               < 2e-2
Shapes cover padding of K to a multiple of 8 (odd D), partial M/N tiles,
and the chain-end MPO bonds (wl = 1).
"""

import numpy as np
import pytest

import oracle as O
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300.utilities import heisenberg_xxz_mpo, j1j2_heisenberg_mpo, FiniteMPO

pytestmark = pytest.mark.gpu

TOL = {"tf32x3": 2e-6, "tf32": 3e-3, "bf16": 2e-2}


def tol(prec, K):
    """3xTF32 is limited by the tensor cores' FP32 accumulation, whose error
    grows with the summed length K (measured ~6e-9 per unit of K); TF32 and
    BF16 are limited by operand rounding."""
    return max(TOL[prec], 1e-8 * K) if prec == "tf32x3" else TOL[prec]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def herm(rng, D, w):
    E = rng.standard_normal((D, w, D))
    return 0.5 * (E + E.transpose(2, 1, 0))


@pytest.mark.parametrize("prec", ["tf32x3", "tf32", "bf16"])
@pytest.mark.parametrize("Dl,Dr", [(8, 8), (13, 21), (64, 64), (100, 37), (256, 256)])
def test_ac2_prime_mixed(prec, Dl, Dr):
    rng = np.random.default_rng(Dl * 1000 + Dr)
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    x = rng.standard_normal((Dl, 2, 2, Dr))
    L, R = herm(rng, Dl, 5), herm(rng, Dr, 5)
    ref = O.ac2_prime(x, W, W, L, R)
    y = fm.ac2_prime(DT.from_numpy(x), W, W, DT.from_numpy(L), DT.from_numpy(R),
                     precision=prec).numpy()
    assert rel(y, ref) < tol(prec, Dl + 5 * Dr), rel(y, ref)


@pytest.mark.parametrize("D", [2048, 1536])
def test_ac2_prime_bf16_large_grids(D):
    """The bench's size and a non-power-of-two one with several waves of GEMM tiles,
    against the device FP64 form (the oracle pins FP64 at the smaller sizes above)."""
    rng = np.random.default_rng(D)
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    x = rng.standard_normal((D, 2, 2, D))
    L, R = herm(rng, D, 5), herm(rng, D, 5)
    args = (DT.from_numpy(x), W, W, DT.from_numpy(L), DT.from_numpy(R))
    ref = fm.ac2_prime(*args, precision="fp64").numpy()
    y = fm.ac2_prime(*args, precision="bf16").numpy()
    assert rel(y, ref) < TOL["bf16"], rel(y, ref)


@pytest.mark.parametrize("prec", ["bf16", "tf32", "tf32x3"])
@pytest.mark.parametrize("Dl,Dr", [(48, 48), (80, 80), (100, 37), (512, 512)])
def test_pair_tile_matches_single_tile(prec, Dl, Dr):
    """The two-CTA 256x256 tile (tcgen05.mma.cta_group::2) against the one-CTA 128x256
    tile on the same inputs.  Both sum the same BF16 (TF32) products in FP32; a different
    summation order may flip the BF16 rounding of a few intermediate elements, so the
    bound between them is 1e-4, far below the BF16 and TF32 bounds.  GEMM 1 is (4 Dr) x (5 Dl), GEMM 2 (4 Dl) x Dr: the sizes leave
    the odd CTA's half of the last tile partly (M = 192, 148, 400; N = 240, 400, 500) and
    wholly (M = 320; N = 48, 80, 37) past the last row or column."""
    from finitemptools_gb300.device import default_handle
    rng = np.random.default_rng(Dl + 7 * Dr)
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    x = rng.standard_normal((Dl, 2, 2, Dr))
    L, R = herm(rng, Dl, 5), herm(rng, Dr, 5)
    args = (DT.from_numpy(x), W, W, DT.from_numpy(L), DT.from_numpy(R))
    h = default_handle()
    y_pair = fm.ac2_prime(*args, precision=prec).numpy()
    h.set_tc_tile("single")
    try:
        y_single = fm.ac2_prime(*args, precision=prec).numpy()
    finally:
        h.set_tc_tile("pair")
    ref = O.ac2_prime(x, W, W, L, R)
    assert rel(y_pair, ref) < tol(prec, Dl + 5 * Dr), rel(y_pair, ref)
    assert rel(y_pair, y_single) < 1e-4, rel(y_pair, y_single)


@pytest.mark.parametrize("prec,D", [("bf16", 512), ("bf16", 1536), ("tf32", 512),
                                    ("tf32x3", 512)])
def test_pair_tail_split_is_deterministic(prec, D):
    """The pair GEMM cuts the tiles of a last, part-filled round along K (GEMM 1 of D=1536
    into 2 pieces; at D=512 GEMM 1 into 2 and GEMM 2 into 4) and adds the partial tiles in
    piece order: repeated applications give identical bits, within the BF16 bound of the
    oracle-pinned FP64 form."""
    rng = np.random.default_rng(D + 3)
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    x = rng.standard_normal((D, 2, 2, D))
    L, R = herm(rng, D, 5), herm(rng, D, 5)
    args = (DT.from_numpy(x), W, W, DT.from_numpy(L), DT.from_numpy(R))
    op = fm.HeffOp("ac2", args[3], args[4], W1=W, W2=W, precision=prec)
    ys = [op(args[0]).numpy() for _ in range(3)]
    assert all(np.array_equal(ys[0], y) for y in ys[1:])
    ref = fm.ac2_prime(*args, precision="fp64").numpy()
    assert rel(ys[0], ref) < tol(prec, 6 * D), rel(ys[0], ref)


@pytest.mark.parametrize("prec", ["tf32x3", "tf32", "bf16"])
def test_ac2_prime_mixed_j1j2_and_boundary(prec):
    rng = np.random.default_rng(7)
    h = j1j2_heisenberg_mpo(1.0, 0.5)
    Ws = FiniteMPO(h, 6)
    x = rng.standard_normal((1, 2, 2, 40))
    L = np.ones((1, 1, 1))
    R = herm(rng, 40, 8)
    ref = O.ac2_prime(x, Ws[0], Ws[1], L, R)
    y = fm.ac2_prime(DT.from_numpy(x), Ws[0], Ws[1], DT.from_numpy(L), DT.from_numpy(R),
                     precision=prec).numpy()
    assert rel(y, ref) < tol(prec, 8 * 40)
    x = rng.standard_normal((72, 2, 2, 48))
    L, R = herm(rng, 72, 8), herm(rng, 48, 8)
    W = h[1].dense()
    ref = O.ac2_prime(x, W, W, L, R)
    y = fm.ac2_prime(DT.from_numpy(x), W, W, DT.from_numpy(L), DT.from_numpy(R),
                     precision=prec).numpy()
    assert rel(y, ref) < tol(prec, 8 * 48 + 72)


@pytest.mark.parametrize("prec", ["tf32x3", "tf32", "bf16"])
def test_ac_and_c_prime_mixed(prec):
    rng = np.random.default_rng(3)
    W = j1j2_heisenberg_mpo()[1].dense()
    x = rng.standard_normal((40, 2, 56))
    L, R = herm(rng, 40, 8), herm(rng, 56, 8)
    y = fm.ac_prime(DT.from_numpy(x), W, DT.from_numpy(L), DT.from_numpy(R), precision=prec)
    assert rel(y.numpy(), O.ac_prime(x, W, L, R)) < tol(prec, 8 * 56)
    C = rng.standard_normal((40, 56))
    yc = fm.c_prime(DT.from_numpy(C), DT.from_numpy(L), DT.from_numpy(R), precision=prec)
    assert rel(yc.numpy(), O.c_prime(C, L, R)) < tol(prec, 8 * 56)


def test_mixed_lanczos_energy_close_to_fp64():
    """Lanczos on the mixed operators (symmetric H_eff): the Ritz value moves
    by the operator error only, and the FP64 Rayleigh quotient of the mixed
    Ritz vector is second order in it."""
    from helpers import xz_mpo, sym_env
    rng = np.random.default_rng(11)
    D = 48
    W = xz_mpo()
    L, R = sym_env(rng, D, 4), sym_env(rng, D, 4)
    x = rng.standard_normal((D, 2, 2, D))
    Ld, Rd = DT.from_numpy(L), DT.from_numpy(R)
    op64 = fm.HeffOp("ac2", Ld, Rd, W1=W, W2=W)
    e64, v64, _, _ = op64.lanczos(DT.from_numpy(x), 60, 1e-12, reorth=True)
    for prec, bound in (("tf32x3", 1e-5), ("tf32", 1e-3), ("bf16", 1e-2)):
        op = fm.HeffOp("ac2", Ld, Rd, W1=W, W2=W, precision=prec)
        e, v, _, _ = op.lanczos(DT.from_numpy(x), 60, 1e-12, reorth=True)
        assert abs(e - e64) < bound * abs(e64), (prec, e, e64)
        hv = op64(v)
        rq = fm.auxiliary.dot(v, hv) / fm.auxiliary.dot(v, v)
        assert abs(rq - e64) < max(bound ** 2, 1e-10) * 100 * abs(e64), (prec, rq, e64)


def _dmrg(L, mpo, D, sweeps, prec, svd, reorth, seed=20):
    rng = np.random.default_rng(seed)
    st = O.randommps(L, 2, 8, rng)
    st, _ = O.canonicalize(st, normalize=True)
    env = fm.environments(FiniteMPO(mpo, L), fm.FiniteMPS.from_numpy(st))
    alg = fm.DMRG2(eig_maxiter=30, eig_tol=1e-12, trunc=fm.MPSTruncation(D, 1e-10),
                   precision=prec, reorth=reorth, svd=svd)
    for _ in range(sweeps):
        Es, delta = fm.sweep_(env, alg)
    return Es, fm.expectation(env.mps, FiniteMPO(mpo, L))


def test_mixed_dmrg2_energy_within_1e8_of_fp64():
    """The spec bar on the XXZ chain (L=20, D=64, 4 sweeps): the state
    found with 3xTF32 contractions, FP64 Lanczos reorthogonalisation and the
    FP64 density-matrix split has an FP64 energy within 1e-8 (relative) of
    the plain FP64 sweep; the density-matrix split alone changes nothing at
    1e-10."""
    h = heisenberg_xxz_mpo(1.0, 1.0, 0.0)
    Es64, E64 = _dmrg(20, h, 64, 4, "fp64", "gesvd", False)
    Esdm, Edm = _dmrg(20, h, 64, 4, "fp64", "dm", False)
    Es3, E3 = _dmrg(20, h, 64, 4, "tf32x3", "dm", True)
    assert abs(Edm - E64) < 1e-10 * abs(E64)
    assert abs(E3 - E64) < 1e-8 * abs(E64)
    # the mixed Ritz values carry the first-order operator error only
    assert abs(Es3[-1] - E64) < 1e-5 * abs(E64)


@pytest.mark.parametrize("prec", ["tf32x3", "tf32", "bf16"])
@pytest.mark.parametrize("Dl,Dr,wl,wr,d", [(1, 2, 1, 8, 2), (13, 21, 5, 5, 2), (64, 48, 8, 8, 2),
                                           (24, 24, 4, 3, 4), (128, 128, 8, 8, 2)])
def test_env_updates_mixed(prec, Dl, Dr, wl, wr, d):
    rng = np.random.default_rng(Dl * 7 + Dr + wl)
    W = rng.standard_normal((wl, d, wr, d)) * (rng.random((wl, 1, wr, 1)) < 0.6)
    A = rng.standard_normal((Dl, d, Dr))
    B = rng.standard_normal((Dl, d, Dr))
    Lh = rng.standard_normal((Dl, wl, Dl))
    Rh = rng.standard_normal((Dr, wr, Dr))
    K = 2 * max(Dl * d, Dr * d)      # the two GEMMs' summed lengths (K1 + K2 <= 2 max)
    gl = fm.updateleft(DT.from_numpy(Lh), DT.from_numpy(A), W, DT.from_numpy(B), prec).numpy()
    assert rel(gl, O.updateleft(Lh, A, W, B)) < tol(prec, K)
    gr = fm.updateright(DT.from_numpy(Rh), DT.from_numpy(A), W, DT.from_numpy(B), prec).numpy()
    assert rel(gr, O.updateright(Rh, A, W, B)) < tol(prec, K)


# ------------------------------------------------------------ complex data
def cherm(rng, D, w):
    E = rng.standard_normal((D, w, D)) + 1j * rng.standard_normal((D, w, D))
    return 0.5 * (E + np.conj(E.transpose(2, 1, 0)))


@pytest.mark.parametrize("prec", ["tf32x3", "tf32", "bf16"])
@pytest.mark.parametrize("Dl,Dr", [(7, 13), (64, 64), (100, 37)])
def test_complex_mixed_forms(prec, Dl, Dr):
    """Complex data on the tensor cores through the real embedding (split
    planes): ac2, ac and c against complex FP64, same bounds as the real forms
    with K doubled (the embedding sums real and imaginary products)."""
    rng = np.random.default_rng(Dl + 7 * Dr)
    W = heisenberg_xxz_mpo(1.0, 0.7, 0.2)[1].dense()
    L, R = cherm(rng, Dl, 5), cherm(rng, Dr, 5)
    dL, dR = DT.from_numpy(L), DT.from_numpy(R)
    x2 = rng.standard_normal((Dl, 2, 2, Dr)) + 1j * rng.standard_normal((Dl, 2, 2, Dr))
    ref = O.ac2_prime(x2, W, W, L, R)
    y = fm.ac2_prime(DT.from_numpy(x2), W, W, dL, dR, precision=prec).numpy()
    assert rel(y, ref) < tol(prec, 2 * (Dl + 5 * Dr)), rel(y, ref)
    x1 = rng.standard_normal((Dl, 2, Dr)) + 1j * rng.standard_normal((Dl, 2, Dr))
    ref = O.ac_prime(x1, W, L, R)
    y = fm.ac_prime(DT.from_numpy(x1), W, dL, dR, precision=prec).numpy()
    assert rel(y, ref) < tol(prec, 2 * (Dl + 5 * Dr)), rel(y, ref)
    C = rng.standard_normal((Dl, Dr)) + 1j * rng.standard_normal((Dl, Dr))
    ref = O.c_prime(C, L, R)
    y = fm.c_prime(DT.from_numpy(C), dL, dR, precision=prec).numpy()
    assert rel(y, ref) < tol(prec, 2 * (Dl + 5 * Dr)), rel(y, ref)


def test_complex_mixed_rejects_complex_mpo():
    rng = np.random.default_rng(5)
    W = heisenberg_xxz_mpo()[1].dense().astype(np.complex128)
    W[0, 0, 1, 1] += 0.1j
    L, R = cherm(rng, 8, 5), cherm(rng, 8, 5)
    x = rng.standard_normal((8, 2, 8)) + 0j
    with pytest.raises(fm.FMPTError):
        fm.ac_prime(DT.from_numpy(x), W, DT.from_numpy(L), DT.from_numpy(R), precision="tf32x3")


def test_tdvp1_complex_mixed_matches_fp64():
    """Config 5's chosen form: TDVP1 with 3xTF32 complex contractions (FP64
    Krylov, QR and environment updates) tracks the FP64 trajectory."""
    rng = np.random.default_rng(40)
    L = 12
    hs = 1.0 + 0.1 * rng.standard_normal(L)
    psi0 = fm.randommps(L, 2, 16, rng, dtype=np.complex128)
    fm.canonicalize_(psi0, normalize=True)
    Z = np.diag([-1.0, 1.0])
    vals = {}
    for prec in ("fp64", "tf32x3"):
        psi = fm.FiniteMPS([A.copy() for A in psi0.data])
        env = fm.environments(fm.tfi_mpo(hs), psi)
        alg = fm.TDVP1(stepsize=-0.05j, D=16, exptol=1e-8, krylovdim=20, precision=prec)
        for _ in range(5):
            fm.sweep_(env, alg)
        vals[prec] = [float(np.real(fm.expectation_local(env.mps, i, Z))) for i in (3, 6, 9)]
    assert np.abs(np.array(vals["tf32x3"]) - np.array(vals["fp64"])).max() < 1e-5


@pytest.mark.parametrize("prec,cplx,D", [("bf16", False, 100), ("tf32x3", False, 256),
                                         ("tf32", False, 37), ("fp64", False, 64),
                                         ("bf16", True, 48), ("bf16", False, 1030),
                                         ("tf32x3", False, 1024), ("bf16", False, 2048)])
def test_ac2_prime_host_matches_device_path(prec, cplx, D):
    """fmpt_ac2_prime_host (host buffers, pipelined transfers for real mixed
    precision) gives the result of copy-in + fmpt_ac2_prime + copy-out: exactly, except
    where it runs GEMM 2 of a mixed-precision operator in column blocks (Dr >= 256).  There the
    pair GEMM cuts the tiles of each launch's part-filled last round along K, a choice
    that depends on the launch's width, so the FP32 sums of those tiles may be ordered
    differently: bound 1e-8 per unit of the summed length K = 2 w D, the FP32 accumulation
    scale the tolerances above use."""
    import torch
    from finitemptools_gb300.derivatives import ac2_prime_host
    rng = np.random.default_rng(D)
    W = heisenberg_xxz_mpo()[1].dense()
    w = W.shape[0]

    def r(*s):
        a = rng.standard_normal(s)
        return a + 1j * rng.standard_normal(s) if cplx else a

    x, L, R = r(D, 2, 2, D), r(D, w, D), r(D, w, D)
    dt = np.complex128 if cplx else np.float64
    ref = fm.ac2_prime(DT.from_numpy(x, dtype=dt), W, W, DT.from_numpy(L, dtype=dt),
                       DT.from_numpy(R, dtype=dt), precision=prec).numpy()
    y = ac2_prime_host(x, W, W, L, R, precision=prec)

    def same(a, b):
        if prec != "fp64" and D >= 256:
            return rel(a, b) < 1e-8 * 2 * w * D
        return np.array_equal(a, b)

    assert same(y, ref)
    if not cplx:
        # page-locked host buffers through the C ABI, as the bench's end-to-end step uses
        from finitemptools_gb300._native import lib, PREC
        h = fm.default_handle()
        px = torch.from_numpy(x.ravel(order="F").copy()).pin_memory()
        pL = torch.from_numpy(L.ravel(order="F").copy()).pin_memory()
        pR = torch.from_numpy(R.ravel(order="F").copy()).pin_memory()
        py = torch.empty(x.size, dtype=torch.float64).pin_memory()
        Wb = np.ascontiguousarray(W.ravel(order="F"))
        h.check(lib().fmpt_ac2_prime_host(h.ptr, 0, PREC[prec], px.data_ptr(), Wb.ctypes.data,
                                          Wb.ctypes.data, pL.data_ptr(), pR.data_ptr(),
                                          py.data_ptr(), D, 2, 2, D, w, w, w))
        assert same(py.numpy().reshape(x.shape, order="F"), ref)
