"""CPU pins of the oracle's discrete TDVP1 adjoint.

The reference has no gradient code; the adjoint is pinned by central finite
differences of the same forward map (exact exponentials) and by a checkpointed
re-run that must give the identical gradient.
"""

import numpy as np
import pytest

from oracle import tdvp_adjoint as TA
from oracle.algorithms import canonicalize, randommps


def _state(L, D, seed):
    rng = np.random.default_rng(seed)
    mps = randommps(L, 2, D, rng, dtype=np.complex128)
    mps, _ = canonicalize(mps, normalize=True)
    h = 1.0 + 0.1 * rng.standard_normal(L)
    return mps, h


def test_qr_adjoint_matches_fd():
    """Thin complex QR with real diag(R): Mbar against finite differences of a
    gauge-invariant loss (Q Q^H and R^H R do not depend on the column phases)."""
    rng = np.random.default_rng(1)
    m, n = 7, 4
    M = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    A = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))

    def loss(M):
        Q, R = np.linalg.qr(M)
        return np.real(np.trace(A @ Q @ Q.conj().T)) + np.real(np.trace(B @ R.conj().T @ R))

    Q, R = np.linalg.qr(M)
    Qbar = (A + A.conj().T) @ Q              # d/dQ of Re tr(A Q Q^H)
    Rbar = R @ (B + B.conj().T)              # d/dR of Re tr(B R^H R)
    Mbar = TA.qr_backward(Q, R, Qbar, Rbar)
    eps = 1e-6
    for (i, j) in [(0, 0), (3, 2), (6, 3)]:
        for unit in (1.0, 1j):
            dM = np.zeros_like(M)
            dM[i, j] = unit * eps
            fd = (loss(M + dM) - loss(M - dM)) / (2 * eps)
            an = np.real(np.conj(Mbar[i, j]) * unit)
            assert abs(fd - an) < 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("L,D,nsteps,site", [(5, 4, 2, 2), (6, 4, 3, 3)])
def test_tdvp1_adjoint_matches_fd(L, D, nsteps, site):
    mps, h = _state(L, D, 3 + L)
    Z = np.diag([-1.0, 1.0])
    val, g = TA.loss_and_grad(h, mps, -0.05j, nsteps, site, Z)
    gfd = TA.fd_grad(h, mps, -0.05j, nsteps, site, Z)
    assert np.linalg.norm(g - gfd) <= 1e-7 * np.linalg.norm(gfd)
