"""CPU pins of the restated projected (excited-state) DMRG (oracle/excited.py):
the overlap storages against dense overlaps, and the first excited energy of
projected DMRG2 / DMRG1 / DMRG1S against exact diagonalisation -- the
reference's own check (test/runtests.jl:495-533 compares the projected DMRG2
and DMRG1S energies with the second ED eigenvalue)."""

import numpy as np

import oracle as O
from oracle import ed
from oracle import excited as OE
from finitemptools_gb300.utilities import tfi_mpo


def _tfi(L, seed):
    rng = np.random.default_rng(seed)
    return 1.5 + 0.2 * rng.standard_normal(L)


def _ground(Ws, L, seed, D=32, sweeps=6):
    rng = np.random.default_rng(seed)
    st, _ = O.canonicalize(O.randommps(L, 2, 4, rng), normalize=True)
    env = O.environments(Ws, st, schur=True)
    for _ in range(sweeps):
        O.dmrg2_sweep(env, O.MPSTruncation(D, 1e-12), 20, 1e-12)
    return env.mps


def test_overlap_storage_is_the_dense_overlap():
    L = 6
    rng = np.random.default_rng(0)
    for dt in (np.float64, np.complex128):
        a = O.randommps(L, 2, 4, rng, dtype=dt)
        b = O.randommps(L, 2, 3, rng, dtype=dt)
        env = OE.ProjectedEnv(tfi_mpo(_tfi(L, 1)).site_tensors(L), a, [b], schur=True)
        cs = env.cstorages[0]
        # the right-initialised chain ends in <a|b> at cs[1] contracted with cs[0]
        full = OE.overlap_updateright(cs[1], a[0], b[0])
        ref = np.vdot(O.mps_to_dense(a), O.mps_to_dense(b))
        assert abs(full[0, 0] - ref) < 1e-12 * max(1.0, abs(ref))
        # the left update chain gives the same number
        h = cs[0]
        for i in range(L):
            h = OE.overlap_updateleft(h, a[i], b[i])
        assert abs(h[0, 0] - ref) < 1e-12 * max(1.0, abs(ref))
        # c_proj of b at a site, contracted with conj(a) there, is <a|b> as well
        env.mps = [A.copy() for A in a]
        for i in range(1, 3):
            env.updateleft_(i)
        p = env.p1(3)
        assert abs(np.vdot(a[2], p) - ref) < 1e-12 * max(1.0, abs(ref))


def test_projected_dmrg_first_excited_energy_matches_ed():
    L = 8
    hs = _tfi(L, 5)
    Ws = tfi_mpo(hs).site_tensors(L)
    H = ed.dense_from_terms(L, 2, ed.tfi_terms(L, hs))
    E = np.linalg.eigvalsh(H)
    gs = _ground(Ws, L, 6)
    assert abs(O.expectation_mpo(gs, Ws, schur=True) - E[0]) < 1e-9
    rng = np.random.default_rng(7)
    st, _ = O.canonicalize(O.randommps(L, 2, 4, rng), normalize=True)
    # DMRG2
    env = OE.ProjectedEnv(Ws, st, [gs], schur=True)
    for _ in range(8):
        Es, _ = OE.pdmrg2_sweep(env, O.MPSTruncation(32, 1e-12), 20, 1e-12)
    assert abs(Es[-1] - E[1]) < 1e-8
    # DMRG1S (the reference's default)
    env = OE.ProjectedEnv(Ws, st, [gs], schur=True)
    for _ in range(10):
        Es, _ = OE.pdmrg1s_sweep(env, O.MPSTruncation(32, 1e-12), 20, 1e-12)
    assert abs(Es[-1] - E[1]) < 1e-8
    # DMRG1 at a fixed bond dimension
    env = OE.ProjectedEnv(Ws, st, [gs], schur=True)
    for _ in range(8):
        Es, _ = OE.pdmrg1_sweep(env, 16, 20, 1e-12)
    assert abs(Es[-1] - E[1]) < 1e-8
    # second excited state: project out both lower states
    env1 = OE.ProjectedEnv(Ws, st, [gs], schur=True)
    for _ in range(8):
        OE.pdmrg2_sweep(env1, O.MPSTruncation(32, 1e-12), 20, 1e-12)
    env2 = OE.ProjectedEnv(Ws, st, [gs, env1.mps], schur=True)
    for _ in range(8):
        Es, _ = OE.pdmrg2_sweep(env2, O.MPSTruncation(32, 1e-12), 20, 1e-12)
    assert abs(Es[-1] - E[2]) < 1e-7
