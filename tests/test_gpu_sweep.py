"""The whole-sweep entry point fmpt_dmrg2_sweep (one C-ABI call per DMRG2 sweep,
algorithms/dmrgexcited.jl:219-223 -> dmrg.jl:89-144) against the Python-driven bond
loop, and the J1-J2 DMRG2 sweep against the oracle.

Bar: the device driver runs the same library calls per bond as the Python driver, so
Ritz values, fidelity deltas and the final tensors are bit-identical; the J1-J2 Ritz
values are within 1e-10 of the oracle's.
"""

import ctypes

import numpy as np
import pytest

import oracle as O
import finitemptools_gb300 as fm
from finitemptools_gb300._native import lib
from finitemptools_gb300.device import to_host_mpo
from finitemptools_gb300.utilities import FiniteMPO, heisenberg_xxz_mpo, j1j2_heisenberg_mpo

pytestmark = pytest.mark.gpu


def _start(L, D0, seed, cplx=False):
    rng = np.random.default_rng(seed)
    st = O.randommps(L, 2, D0, rng, dtype=np.complex128 if cplx else np.float64)
    st, _ = O.canonicalize(st, normalize=True)
    return st


@pytest.mark.parametrize("cplx,svd,prec", [(False, "gesvd", "fp64"), (False, "dm", "fp64"),
                                           (False, "dm", "tf32x3"), (True, "gesvd", "fp64")])
def test_device_sweep_bit_identical_to_python_driver(cplx, svd, prec):
    L = 12
    h = heisenberg_xxz_mpo(1.0, 1.0, 0.3)
    st = _start(L, 4, 7, cplx)
    envs = {}
    for drv in ("python", "device"):
        envs[drv] = fm.environments(h, fm.FiniteMPS.from_numpy(st))
    algs = {drv: fm.DMRG2(eig_maxiter=20, eig_tol=1e-12, trunc=fm.MPSTruncation(24, 1e-10),
                          svd=svd, precision=prec, driver=drv, verbosity=0)
            for drv in ("python", "device")}
    for _ in range(3):
        Ep, dp = fm.sweep_(envs["python"], algs["python"])
        Ed, dd = fm.sweep_(envs["device"], algs["device"])
        assert len(Ed) == 2 * L - 3
        assert Ed == Ep
        assert dd == dp
    mp, md = envs["python"].mps, envs["device"].mps
    for i in range(1, L + 1):
        assert md[i].shape == mp[i].shape
        assert np.array_equal(md[i].numpy(), mp[i].numpy())
    for b in range(2, L + 1):
        assert np.array_equal(md.s[b].numpy(), mp.s[b].numpy())
    for b in range(1, L + 2):
        assert np.array_equal(envs["device"].hstorage[b].numpy(),
                              envs["python"].hstorage[b].numpy())
    # the driver keeps working on the grown buffers: a Python sweep after device sweeps
    Ep, _ = fm.sweep_(envs["python"], algs["python"])
    Ed, _ = fm.sweep_(envs["device"], algs["python"])
    assert Ed == Ep


@pytest.mark.parametrize("driver", ["python", "device"])
def test_j1j2_L20_dmrg2_oracle_parity(driver):
    """FP64 DMRG2 on the J1-J2 chain (J2 = 0.5, w = 8 Schur MPO), L = 20: every Ritz value
    of two sweeps within 1e-10 of the oracle's."""
    L = 20
    h = j1j2_heisenberg_mpo(1.0, 0.5)
    st = _start(L, 8, 21)
    env_o = O.environments(FiniteMPO(h, L), st)
    env_d = fm.environments(FiniteMPO(h, L), fm.FiniteMPS.from_numpy(st))
    alg = fm.DMRG2(eig_maxiter=20, eig_tol=1e-12, trunc=fm.MPSTruncation(32, 1e-10),
                   driver=driver, verbosity=0)
    for _ in range(2):
        Eo, do = O.dmrg2_sweep(env_o, O.MPSTruncation(32, 1e-10), 20, 1e-12)
        Ed, dd = fm.sweep_(env_d, alg)
        assert len(Eo) == len(Ed) == 2 * L - 3
        assert np.max(np.abs(np.array(Eo) - np.array(Ed))) < 1e-10
        assert abs(do - dd) < 1e-8


def test_device_sweep_rejects_buffers_that_do_not_fit():
    """A site buffer smaller than its tensor is refused before anything runs."""
    L = 4
    st = _start(L, 2, 3)
    psi = fm.FiniteMPS.from_numpy(st)
    env = fm.environments(heisenberg_xxz_mpo(1.0, 1.0, 0.0), psi)
    h = psi.handle
    phys = [2] * L
    bond = [psi[1].shape[0]] + [psi[i].shape[2] for i in range(1, L + 1)]
    wb = [env.mpo[1].shape[0]] + [env.mpo[i].shape[2] for i in range(1, L + 1)]
    caps = [bond[i] * 2 * bond[i + 1] for i in range(L)]
    caps[1] -= 1
    Ws = [to_host_mpo(W, np.float64) for W in env.mpo]
    arr, earr = ctypes.c_void_p * L, ctypes.c_void_p * (L + 1)
    en = (ctypes.c_double * (2 * L - 3))()
    dl = ctypes.c_double()
    st_ = lib().fmpt_dmrg2_sweep(
        h.ptr, 0, 0, 0, L, (ctypes.c_int * L)(*phys), (ctypes.c_int * (L + 1))(*bond),
        arr(*[psi[i].ptr for i in range(1, L + 1)]), (ctypes.c_int64 * L)(*caps),
        earr(*[env.hstorage[b].ptr for b in range(1, L + 2)]),
        (ctypes.c_int64 * (L + 1))(*[bond[b] * wb[b] * bond[b] for b in range(L + 1)]),
        arr(*[w.ctypes.data for w in Ws]), (ctypes.c_int * (L + 1))(*wb), None, 8, 1e-10, 10,
        1e-12, 0, 0, en, ctypes.byref(dl))
    assert st_ == -2
    assert b"does not fit" in lib().fmpt_last_error(h.ptr)
