"""CPU pins of the U(1) block-sparse oracle and of the host-side sector
bookkeeping (no GPU needed).

The reference's symmetric path has no stored vectors; the oracle is pinned by
exact facts: the per-block contraction equals the dense contraction on the
charge-sorted tensors (whose forbidden entries stay exactly zero), the
per-sector singular values are the singular values of the whole two-site
matrix, and U(1) DMRG2 reaches the exact ground energy of the Sz sector.
"""

import numpy as np
import pytest

import oracle as O
from oracle import u1 as OU
from oracle.ed import xxz_ground_energy
from finitemptools_gb300.utilities import heisenberg_xxz_mpo

QP = [0, 1]


def _bond(L, N, D, site, seed):
    rng = np.random.default_rng(seed)
    Ws = heisenberg_xxz_mpo(1.0, 0.7, 0.3).site_tensors(L)
    qw = OU.channel_charges(Ws, QP)
    mps, legs = OU.random_u1_state(L, N, D, QP, rng)
    Vl, Vr = legs[site - 1], legs[site + 1]
    X = np.tensordot(mps[site - 1], mps[site], axes=([2], [0]))
    Lm = rng.standard_normal((Vl.dim, 5, Vl.dim)) * OU.allowed_env(Vl, qw[site - 1])
    Rm = rng.standard_normal((Vr.dim, 5, Vr.dim)) * OU.allowed_env(Vr, qw[site + 1])
    return Ws, qw, mps, legs, X, Lm, Rm


def test_channel_charges_heisenberg():
    """identity, S+, S-, Z, final: charges 0, +1, -1, 0, 0 on every bond."""
    qw = OU.channel_charges(heisenberg_xxz_mpo().site_tensors(6), QP)
    assert all(list(q) == [0, 1, -1, 0, 0] for q in qw)


@pytest.mark.parametrize("L,N,D,site", [(8, 4, 6, 3), (10, 5, 12, 4), (10, 3, 20, 7)])
def test_blocks_equal_dense(L, N, D, site):
    Ws, qw, mps, legs, X, Lm, Rm = _bond(L, N, D, site, L * 7 + D)
    Vl, Vr = legs[site - 1], legs[site + 1]
    Y1 = O.ac2_prime(X, Ws[site - 1], Ws[site], Lm, Rm)
    Y2 = OU.ac2_prime_blocks(X, Ws[site - 1], Ws[site], Lm, Rm, Vl, Vr, QP, QP, qw[site - 1],
                             qw[site + 1])
    assert np.abs(Y1 - Y2).max() <= 1e-13 * np.abs(Y1).max()
    allowed = OU.unpack2(OU.pack2(np.ones_like(Y1), Vl, Vr, QP, QP), Vl, Vr, QP, QP)
    assert np.all(Y1[allowed == 0] == 0.0)
    assert np.array_equal(OU.unpack2(OU.pack2(Y1, Vl, Vr, QP, QP), Vl, Vr, QP, QP), Y1)


def test_split_spectrum_is_dense_svd():
    Ws, qw, mps, legs, X, Lm, Rm = _bond(10, 5, 16, 5, 3)
    Vl, Vr = legs[4], legs[6]
    A, S, B, Vm, err = OU.u1_split(X, Vl, Vr, QP, QP, O.MPSTruncation(10000, 0.0), 0)
    sd = np.linalg.svd(X.reshape(Vl.dim * 2, 2 * Vr.dim, order="F"), compute_uv=False)
    sd = sd[:len(S)] / np.linalg.norm(sd)
    assert np.abs(np.sort(S)[::-1] - sd).max() < 1e-13
    assert err < 1e-12
    # untruncated split reproduces the normalised two-site tensor
    X2 = np.tensordot(A, B, axes=([2], [0]))
    assert np.linalg.norm(X2 - X / np.linalg.norm(X)) < 1e-12


def test_split_truncation_rule():
    """Cross-sector rule: keep the globally largest maxD values."""
    Ws, qw, mps, legs, X, Lm, Rm = _bond(10, 5, 16, 5, 4)
    Vl, Vr = legs[4], legs[6]
    full = OU.u1_split(X, Vl, Vr, QP, QP, O.MPSTruncation(10000, 0.0), 0)[1]
    A, S, B, Vm, err = OU.u1_split(X, Vl, Vr, QP, QP, O.MPSTruncation(7, 0.0), 0)
    top = np.sort(full)[::-1][:7]
    assert Vm.dim == 7
    assert np.allclose(np.sort(S)[::-1], top / np.linalg.norm(top), atol=1e-13)
    assert np.isclose(err, np.linalg.norm(np.sort(full)[::-1][7:]) * np.linalg.norm(
        OU.pack2(X, Vl, Vr, QP, QP)), rtol=1e-10)


def test_u1_dmrg2_oracle_matches_ed():
    L, N = 10, 5
    Ws = heisenberg_xxz_mpo().site_tensors(L)
    mps, legs = OU.random_u1_state(L, N, 8, QP, np.random.default_rng(1))
    env = OU.U1OracleEnv(Ws, mps, legs, QP, schur=True)
    env.right_canonicalize()
    for _ in range(3):
        Es, delta = OU.u1_dmrg2_sweep(env, O.MPSTruncation(40, 1e-12), 10, 1e-12)
    assert abs(Es[-1] - xxz_ground_energy(L, nup=N)) < 1e-10


def test_host_packed_size_matches_oracle():
    """fmpt_u1_twosite_size runs on the host (no GPU) and must agree with the
    oracle's packed layout."""
    from finitemptools_gb300.u1 import U1Space, u1_twosite_size
    Ws, qw, mps, legs, X, Lm, Rm = _bond(12, 6, 33, 6, 9)
    Vl, Vr = legs[5], legs[7]
    n = u1_twosite_size(U1Space(Vl.items()), U1Space(Vr.items()), QP, QP)
    assert n == OU.pack2(X, Vl, Vr, QP, QP).size


def test_product_generator_matches_oracle():
    """The synthetic U(1) states of the product and of the oracle are the same
    draws (same legs, same blocks), so parity runs start from one state."""
    from finitemptools_gb300.u1 import random_u1_tensors
    t1, s1 = random_u1_tensors(16, 8, 24, (0, 1), 5)
    t2, s2 = OU.random_u1_state(16, 8, 24, QP, np.random.default_rng(5))
    assert [s.charges for s in s1] == [tuple(l.charges) for l in s2]
    assert [s.dims for s in s1] == [tuple(l.dims) for l in s2]
    assert all(np.array_equal(a, b) for a, b in zip(t1, t2))


def test_channel_charges_reject_nonsymmetric():
    from finitemptools_gb300.u1 import mpo_channel_charges
    Ws = heisenberg_xxz_mpo().site_tensors(4)
    Ws[1] = Ws[1].copy()
    Ws[1][0, 0, 1, 0] = 0.5          # S+ channel on a diagonal entry: charge not conserved
    with pytest.raises(ValueError):
        mpo_channel_charges(Ws, (0, 1))
