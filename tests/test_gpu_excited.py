"""Projected (excited-state) DMRG on the device (finitemptools_gb300.excited and
fmpt_op_set_projectors) against the oracle's restatement (oracle/excited.py)
and exact diagonalisation."""

import numpy as np
import pytest

import oracle as O
from oracle import ed
from oracle import excited as OE
from oracle.core import ac2_prime
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300.utilities import tfi_mpo

pytestmark = pytest.mark.gpu


def _tfi(L, seed):
    rng = np.random.default_rng(seed)
    return 1.5 + 0.2 * rng.standard_normal(L)


def _up(mps, dtype=None):
    return fm.FiniteMPS([DT.from_numpy(A, dtype=dtype) for A in mps])


def _rel(a, b):
    return np.abs(a - b).max() / max(1e-300, np.abs(b).max())


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_overlap_transfers_and_projections(dt):
    rng = np.random.default_rng(1)

    def r(*s):
        x = rng.standard_normal(s)
        return x + 1j * rng.standard_normal(s) if dt == np.complex128 else x

    def g(x):
        return DT.from_numpy(x, dtype=dt)

    A, B = r(5, 2, 7), r(3, 2, 4)
    hl0 = r(5, 3)
    assert _rel(fm.overlap_updateleft(g(hl0), g(A), g(B)).numpy(),
                OE.overlap_updateleft(hl0, A, B)) < 1e-13
    hr = r(7, 4)
    assert _rel(fm.overlap_updateright(g(hr), g(A), g(B)).numpy(),
                OE.overlap_updateright(hr, A, B)) < 1e-13
    x, cl, cr = r(3, 2, 4), r(5, 3), r(7, 4)
    assert _rel(fm.c_proj(g(x), g(cl), g(cr)).numpy(), OE.c_proj(x, cl, cr)) < 1e-13
    x1, x2 = r(3, 2, 6), r(6, 2, 4)
    assert _rel(fm.c2_proj(g(x1), g(x2), g(cl), g(cr)).numpy(),
                OE.c2_proj(x1, x2, cl, cr)) < 1e-13
    # H_eff composed with _project! inside the library, two projectors in order
    W = [np.asarray(Wi) for Wi in tfi_mpo(_tfi(4, 2)).site_tensors(4)]
    W1, W2 = W[1].astype(dt), W[2].astype(dt)
    w = W1.shape[0]
    hl, hrr = r(5, w, 5), r(7, w, 7)
    xx = r(5, 2, 2, 7)
    ps = [r(5, 2, 2, 7), r(5, 2, 2, 7)]
    op = fm.HeffOp("ac2", g(hl), g(hrr), W1=W1, W2=W2, dtype=dt)
    op.set_projectors([g(p) for p in ps])
    y = op(g(xx)).numpy()
    assert _rel(y, OE.project(ac2_prime(xx, W1, W2, hl, hrr), ps)) < 1e-12
    # the host-side _project! on a device vector
    z = fm.project_(g(xx), [g(p) for p in ps]).numpy()
    assert _rel(z, OE.project(xx, ps)) < 1e-13
    # removing the projectors restores the plain operator
    op.set_projectors([])
    assert _rel(op(g(xx)).numpy(), ac2_prime(xx, W1, W2, hl, hrr)) < 1e-12


def _paired(Ws):
    """Two neighbouring spins as one d=4 site: Wp[wl,(s1 s2)',wr,(s1 s2)] (the
    same Hamiltonian, so the same spectrum)."""
    out = []
    for W1, W2 in zip(Ws[0::2], Ws[1::2]):
        wl, d, _, _ = W1.shape
        wr = W2.shape[2]
        t = np.einsum("aibj,bkcl->aikcjl", W1, W2)
        out.append(t.reshape(wl, d * d, wr, d * d, order="F"))
    return out


def _ground_state(Ws, Lp):
    rng = np.random.default_rng(6)
    st, _ = O.canonicalize(O.randommps(Lp, 4, 4, rng), normalize=True)
    env = O.environments(Ws, st)
    for _ in range(6):
        O.dmrg2_sweep(env, O.MPSTruncation(32, 1e-12), 20, 1e-12)
    return env.mps


@pytest.mark.parametrize("algo", ["dmrg2", "dmrg1s", "dmrg1"])
def test_projected_dmrg_matches_oracle_and_ed(algo):
    """TFI chain of 8 spins grouped into 4 sites of d=4, first excited state.
    eig_maxiter is the reference default 10, below every local dimension (16 at
    the edges): _project! is an exact projection only for |p| = 1, and a
    Lanczos run past the dimension of its space amplifies rounding, which makes
    the reference algorithm itself machine-dependent there."""
    L = 8
    hs = _tfi(L, 5)
    Ws = _paired(fm.FiniteMPO(tfi_mpo(hs), L))
    Lp = len(Ws)
    E = np.linalg.eigvalsh(ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs)))
    gs = _ground_state(Ws, Lp)
    rng = np.random.default_rng(7)
    st, _ = O.canonicalize(O.randommps(Lp, 4, 4, rng), normalize=True)
    env_o = OE.ProjectedEnv(Ws, st, [gs])
    env_g = fm.environments(Ws, _up(st), [_up(gs)])
    assert isinstance(env_g, fm.ProjectedExpectationCache)
    tr_o = O.MPSTruncation(32, 1e-12)
    if algo == "dmrg2":
        alg = fm.DMRG2(eig_maxiter=10, eig_tol=1e-12, trunc=fm.MPSTruncation(32, 1e-12),
                       verbosity=0)
    elif algo == "dmrg1s":
        alg = fm.DMRG1S(eig_maxiter=10, eig_tol=1e-12, trunc=fm.MPSTruncation(32, 1e-12),
                        verbosity=0)
    else:
        alg = fm.DMRG1(D=16, eig_maxiter=10, eig_tol=1e-12, verbosity=0)
    for _ in range(10):
        if algo == "dmrg2":
            Eo, _ = OE.pdmrg2_sweep(env_o, tr_o, 10, 1e-12)
        elif algo == "dmrg1s":
            Eo, _ = OE.pdmrg1s_sweep(env_o, tr_o, 10, 1e-12)
        else:
            Eo, _ = OE.pdmrg1_sweep(env_o, 16, 10, 1e-12)
        Eg, _ = fm.sweep_(env_g, alg)
        assert len(Eg) == len(Eo)
        assert np.abs(np.asarray(Eg) - np.asarray(Eo)).max() < 1e-9 * abs(E[1])
    assert abs(Eg[-1] - E[1]) < 1e-8
    psi = O.mps_to_dense([env_g.mps[i].numpy() for i in range(1, Lp + 1)])
    assert abs(np.vdot(O.mps_to_dense(gs), psi)) < 1e-6
