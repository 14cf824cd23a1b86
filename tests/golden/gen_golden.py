"""Generates the committed golden fixtures from the CPU oracle and exact
diagonalisation (run from the repository root: python tests/golden/gen_golden.py).

The reference (Julia) cannot run in this environment; these fixtures pin the
oracle's outputs so GPU tests on a machine without the reference compare
against fixed numbers, and hold the exact-diagonalisation energies that are
too slow to recompute in every test run.
"""

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from oracle import ed  # noqa: E402
from finitemptools_gb300.utilities import heisenberg_xxz_mpo  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    energies = {
        # spin-1/2 XXZ (Pauli convention of utilities/models.jl), open chain
        "xxz_L20_J1_Jzz1_hz0": ed.xxz_ground_energy(20, 1.0, 1.0, 0.0),
        "j1j2_L16_J1_1_J2_0.5": ed.j1j2_ground_energy(16, 1.0, 0.5),
        "xx_L200_free_fermion": ed.xx_free_fermion_energy(200, 1.0),
    }
    with open(os.path.join(OUT, "exact_energies.json"), "w") as f:
        json.dump(energies, f, indent=1)

    # one two-site H_eff*x case (D=12, Heisenberg Schur W, Hermitian L/R)
    rng = np.random.default_rng(2024)
    D, w = 12, 5
    x = rng.standard_normal((D, 2, 2, D))
    L = rng.standard_normal((D, w, D))
    R = rng.standard_normal((D, w, D))
    L = 0.5 * (L + np.transpose(L, (2, 1, 0)))
    R = 0.5 * (R + np.transpose(R, (2, 1, 0)))
    W = heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1].dense()
    y = O.ac2_prime(x, W, W, L, R)
    np.savez_compressed(os.path.join(OUT, "ac2_D12.npz"), x=x, L=L, R=R, W=W, y=y)
    print(json.dumps(energies, indent=1))


if __name__ == "__main__":
    main()
