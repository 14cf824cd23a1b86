"""The FP64-accurate tensor-core engine (Ozaki scheme on BF16 digit planes).

Bar: the same 1e-12 relative (Frobenius) parity with the oracle as the CUDA-core FP64 path,
at the microbenchmark sizes of the two-site H_eff*x (D = 256, 512) and on the environment
updates; GEMMs of integer-valued operands whose exact product is representable come out
bit-exact (every digit product is summed exactly in FP32); Inf/NaN rows propagate.
Each test checks through the device profiler that the tensor-core kernel really ran.
"""

import numpy as np
import pytest

import oracle as O
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300.auxiliary import gemm
from finitemptools_gb300.utilities import heisenberg_xxz_mpo, j1j2_heisenberg_mpo

pytestmark = pytest.mark.gpu

TC_GEMM = 0      # FMPT_K_TC_GEMM


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture
def tc_handle():
    h = fm.default_handle()
    h.set_f64_engine("tensor_cores")
    h.profile(True)
    h.profile_read(TC_GEMM)
    yield h
    h.profile(False)
    h.set_f64_engine("cuda_cores")


def tc_launches(h):
    n, _ = h.profile_read(TC_GEMM)
    return n


def opm(A, t):
    return {"N": A, "T": A.T, "C": A.conj().T, "R": A.conj()}[t]


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("C", "R")])
@pytest.mark.parametrize("m,n,k", [(1000, 777, 1500), (300, 1290, 2600)])
def test_gemm_matches_fp64(tc_handle, cplx, ta, tb, m, n, k):
    rng = np.random.default_rng(m + n + k + 7 * cplx)

    def mat(r, c):
        a = rng.standard_normal((r, c)) * np.exp(rng.standard_normal((r, 1)))
        return a + 1j * rng.standard_normal((r, c)) if cplx else a

    A = mat(m, k) if ta in ("N", "R") else mat(k, m)
    B = mat(k, n) if tb in ("N", "R") else mat(n, k)
    ref = opm(A, ta) @ opm(B, tb)
    dA, dB = DT.from_numpy(A, tc_handle), DT.from_numpy(B, tc_handle)
    C = gemm(dA, dB, (m, n), m, n, k, ta, tb, lda=A.shape[0], ldb=B.shape[0])
    assert tc_launches(tc_handle) >= 1
    # the digits of an entry are taken relative to its row's (column's) largest entry; the
    # operands here span about e^+-3 along K (ta / tb = T scale the K index), where 8
    # digits (48 bits) measured 6e-13 and the 9 digits (54 bits) about 1e-15
    assert rel(C.numpy(), ref) < 1e-13


@pytest.mark.parametrize("cplx", [False, True])
def test_gemm_alpha_beta_and_small_tile_counts(tc_handle, cplx):
    """beta != 0 and a complex alpha run the piece-sum path; a 2 x 2 tile problem splits
    its digit products over several clusters (level sets and K chunks)."""
    rng = np.random.default_rng(11)
    m, n, k = 500, 300, 4100
    A = rng.standard_normal((m, k)) + (1j * rng.standard_normal((m, k)) if cplx else 0)
    B = rng.standard_normal((k, n)) + (1j * rng.standard_normal((k, n)) if cplx else 0)
    C0 = rng.standard_normal((m, n)) + (1j * rng.standard_normal((m, n)) if cplx else 0)
    alpha, beta = (0.5 - 0.25j, 2.0 + 1j) if cplx else (-1.5, 0.75)
    ref = alpha * (A @ B) + beta * C0
    dC = DT.from_numpy(C0, tc_handle)
    gemm(DT.from_numpy(A, tc_handle), DT.from_numpy(B, tc_handle), (m, n), m, n, k,
         alpha=alpha, beta=beta, C=dC)
    assert tc_launches(tc_handle) >= 1
    assert rel(dC.numpy(), ref) < 1e-13


def test_gemm_exact_on_integer_grids(tc_handle):
    """Entries j/64 with |j| <= 63 and all of one sign: the digit sums grow as large as
    same-sign entries make them, the exact product is a multiple of 2^-12 below 2^12,
    representable in FP64, and the tensor-core result must equal it bit for bit."""
    rng = np.random.default_rng(3)
    m, n, k = 768, 640, 2048
    A = rng.integers(1, 64, size=(m, k)) / 64.0
    B = -rng.integers(1, 64, size=(k, n)) / 64.0
    exact = (A * 64).astype(np.int64) @ (B * 64).astype(np.int64) / 4096.0
    C = gemm(DT.from_numpy(A, tc_handle), DT.from_numpy(B, tc_handle), (m, n), m, n, k)
    assert tc_launches(tc_handle) >= 1
    assert np.array_equal(C.numpy(), exact)


def test_gemm_nonfinite_rows_propagate(tc_handle):
    rng = np.random.default_rng(4)
    m, n, k = 512, 512, 1024
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n))
    A[5, 17] = np.nan
    A[9, 3] = np.inf
    C = gemm(DT.from_numpy(A, tc_handle), DT.from_numpy(B, tc_handle), (m, n), m, n, k).numpy()
    assert tc_launches(tc_handle) >= 1
    assert np.isnan(C[5]).all() and np.isnan(C[9]).all()
    ok = np.ones(m, bool)
    ok[[5, 9]] = False
    assert rel(C[ok], A[ok] @ B) < 1e-13


def test_small_gemm_stays_on_cuda_cores(tc_handle):
    """Below the cost model's crossover the FP64 engine keeps the CUDA-core kernel."""
    rng = np.random.default_rng(5)
    A, B = rng.standard_normal((40, 30)), rng.standard_normal((30, 20))
    C = gemm(DT.from_numpy(A, tc_handle), DT.from_numpy(B, tc_handle), (40, 20), 40, 20, 30)
    assert tc_launches(tc_handle) == 0
    assert rel(C.numpy(), A @ B) < 1e-14


def _workload(D, w, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((D, 2, 2, D))
    L = rng.standard_normal((D, w, D))
    R = rng.standard_normal((D, w, D))
    L = 0.5 * (L + L.transpose(2, 1, 0))
    R = 0.5 * (R + R.transpose(2, 1, 0))
    return x, L, R


@pytest.mark.parametrize("D,model", [(256, "xxz"), (512, "xxz"), (256, "j1j2"), (512, "j1j2"),
                                     (1024, "xxz")])
@pytest.mark.parametrize("prec", ["fp64", "fp64_tc"])
def test_ac2_prime_oracle_parity_config_sizes(D, model, prec):
    """Two-site H_eff*x at the microbenchmark sizes, Heisenberg (w=5) and J1-J2 (w=8)
    Schur MPOs, both FP64 forms against the oracle at 1e-12."""
    W = (heisenberg_xxz_mpo(1.0, 1.0, 0.0) if model == "xxz"
         else j1j2_heisenberg_mpo(1.0, 0.5))[1].dense()
    w = W.shape[0]
    x, L, R = _workload(D, w, D + w)
    ref = O.ac2_prime(x, W, W, L, R)
    h = fm.default_handle()
    h.profile(True)
    h.profile_read(TC_GEMM)
    y = fm.ac2_prime(DT.from_numpy(x), W, W, DT.from_numpy(L), DT.from_numpy(R),
                     precision=prec).numpy()
    n = tc_launches(h)
    h.profile(False)
    assert (n >= 1) == (prec == "fp64_tc")
    assert rel(y, ref) < 1e-12


@pytest.mark.parametrize("cplx", [False, True])
def test_ac_prime_and_env_updates_fp64_tc(cplx):
    rng = np.random.default_rng(21 + cplx)
    D, w, d = 384, 5, 2
    W = heisenberg_xxz_mpo(1.0, 0.6, 0.2)[1].dense()

    def r(*s):
        a = rng.standard_normal(s)
        return a + 1j * rng.standard_normal(s) if cplx else a

    x, L, R = r(D, d, D), r(D, w, D), r(D, w, D)
    A, B = r(D, d, D), r(D, d, D)
    y = fm.ac_prime(DT.from_numpy(x), W, DT.from_numpy(L), DT.from_numpy(R),
                    precision="fp64_tc").numpy()
    assert rel(y, O.ac_prime(x, W, L, R)) < 1e-12
    hl = fm.updateleft(DT.from_numpy(L), DT.from_numpy(A), W, DT.from_numpy(B),
                       precision="fp64_tc").numpy()
    assert rel(hl, O.updateleft(L, A, W, B)) < 1e-12
    hr = fm.updateright(DT.from_numpy(R), DT.from_numpy(A), W, DT.from_numpy(B),
                        precision="fp64_tc").numpy()
    assert rel(hr, O.updateright(R, A, W, B)) < 1e-12


def test_lanczos_fp64_tc_matches_fp64():
    """The plain Lanczos on the tensor-core FP64 operator reproduces the CUDA-core FP64
    eigenvalue (the recurrence sees only FP64-accurate products)."""
    from tests.helpers import sym_env, xz_mpo
    rng = np.random.default_rng(8)
    D = 320
    W = xz_mpo()
    L, R = sym_env(rng, D, 4), sym_env(rng, D, 4)
    x0 = rng.standard_normal((D, 2, 2, D))
    Ld, Rd, xd = DT.from_numpy(L), DT.from_numpy(R), DT.from_numpy(x0)
    E64 = fm.HeffOp("ac2", Ld, Rd, W1=W, W2=W, precision="fp64").lanczos(xd, 20, 1e-12)[0]
    Etc = fm.HeffOp("ac2", Ld, Rd, W1=W, W2=W, precision="fp64_tc").lanczos(xd, 20, 1e-12)[0]
    assert abs(Etc - E64) < 1e-11 * abs(E64)
