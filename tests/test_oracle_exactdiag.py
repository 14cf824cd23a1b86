"""CPU pins of the restated ExactFiniteMPS exact diagonalisation and exact time
evolution (oracle/exactdiag.py) against dense linear algebra, and of the
product's host-side bond bookkeeping (max_bond_dimensions, _find_center)
against the restatement."""

import numpy as np
import pytest

import oracle as O
from oracle import ed
from oracle import exactdiag as OX
from finitemptools_gb300 import exactdiag as PX
from finitemptools_gb300.utilities import FiniteMPO, heisenberg_xxz_mpo, tfi_mpo


@pytest.mark.parametrize("physdims", [[2] * 20, [2] * 7, [3, 2, 4, 2, 3], [4, 4, 4, 4], [2]])
def test_bond_dimensions_and_center(physdims):
    assert PX.max_bond_dimensions(physdims) == OX.max_bond_dimensions(physdims)
    assert PX.find_center(PX.max_bond_dimensions(physdims)) == \
        OX.find_center(OX.max_bond_dimensions(physdims))
    out, left, right, mid = OX.side_tensors(physdims)
    assert left * physdims[mid - 1] * right == int(np.prod(physdims))
    for i, A in enumerate(out):
        if A is None:
            continue
        M = A.reshape(A.shape[0] * A.shape[1], A.shape[2], order="F") if i < mid - 1 else \
            A.reshape(A.shape[0], A.shape[1] * A.shape[2], order="F")
        G = M.T @ M if i < mid - 1 else M @ M.T
        assert np.array_equal(G, np.eye(G.shape[0]))


def test_exact_diagonalization_matches_dense():
    L = 8
    rng = np.random.default_rng(3)
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    Ws = FiniteMPO(tfi_mpo(hs), L)
    E = np.linalg.eigvalsh(ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs)))
    vals, states, mid = OX.exact_diagonalization(Ws, num=3)
    assert np.abs(vals - E[:3]).max() < 1e-10
    # the Schur form with its boundary vectors gives the same spectrum
    vals2, _, _ = OX.exact_diagonalization(heisenberg_xxz_mpo().site_tensors(L), num=2,
                                           schur=True)
    assert abs(vals2[0] - ed.xxz_ground_energy(L)) < 1e-10


def test_exact_mps_and_time_evolution_match_dense():
    L, t = 7, -0.3j
    rng = np.random.default_rng(5)
    hs = 1.0 + 0.2 * rng.standard_normal(L)
    Ws = FiniteMPO(tfi_mpo(hs), L)
    psi = O.randommps(L, 2, 3, rng, dtype=np.complex128)
    ex, mid = OX.exact_mps_from(psi)
    assert np.abs(O.mps_to_dense(ex) - O.mps_to_dense(psi)).max() < 1e-13
    out = OX.exact_timeevolution(Ws, t, ex, mid)
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    ref = ed.exact_evolution(H, O.mps_to_dense(psi), t)
    assert np.abs(O.mps_to_dense(out) - ref).max() < 1e-10
