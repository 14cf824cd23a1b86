"""Shared test inputs."""

import numpy as np


def xz_mpo(J=1.0, h=0.3):
    """A w=4 Schur MPO whose every (w, w') block is a real symmetric matrix
    (J X X + J Z Z + h Z): with per-channel symmetric environments the
    effective Hamiltonian is symmetric, so Lanczos is meaningful on random
    environments."""
    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    Z = np.array([[-1.0, 0.0], [0.0, 1.0]])
    I = np.eye(2)
    W = np.zeros((4, 2, 4, 2))
    W[0, :, 0, :] = I
    W[0, :, 1, :] = J * X
    W[0, :, 2, :] = J * Z
    W[0, :, 3, :] = h * Z
    W[1, :, 3, :] = X
    W[2, :, 3, :] = Z
    W[3, :, 3, :] = I
    return W


def sym_env(rng, D, w, cplx=False):
    E = rng.standard_normal((D, w, D))
    if cplx:
        E = E + 1j * rng.standard_normal((D, w, D))
    return 0.5 * (E + np.conj(E.transpose(2, 1, 0)))
