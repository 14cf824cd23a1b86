"""Parity of the device TDVP1 adjoint (finitemptools_gb300.adjoint) with the
oracle's FP64 adjoint and with central finite differences of the device
forward map.

Bar: gradients within 1e-6 relative of central differences (step 1e-5) and of
the oracle's plain FP64 adjoint; building blocks at 1e-11.
"""

import numpy as np
import pytest
import scipy.linalg

import oracle as O
from oracle import tdvp_adjoint as TA
from oracle.algorithms import canonicalize, randommps
import finitemptools_gb300 as fm
from finitemptools_gb300 import DeviceTensor as DT
from finitemptools_gb300 import adjoint as AD

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def crand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_qr_adjoint_kernel():
    rng = np.random.default_rng(2)
    m, n = 12, 5
    M = crand(rng, (m, n))
    dM = DT.from_numpy(M)
    Q, R = fm.leftorth(dM, m, n)
    Qh, Rh = Q.numpy(), R.numpy()
    assert np.abs(np.imag(np.diag(Rh))).max() < 1e-14        # real diag(R): the adjoint's gauge
    Qb, Rb = crand(rng, (m, n)), crand(rng, (n, n))
    Mb = AD.qr_adjoint(Q, R, DT.from_numpy(Qb), DT.from_numpy(Rb), m, n).numpy()
    assert rel(Mb, TA.qr_backward(Qh, Rh, Qb, Rb)) < 1e-11


def test_wgrad_and_swap13():
    rng = np.random.default_rng(3)
    Dl, d, Dr, wl, wr = 5, 2, 7, 3, 4
    a, b = crand(rng, (Dl, d, Dr)), crand(rng, (Dl, d, Dr))
    L, R = crand(rng, (Dl, wl, Dl)), crand(rng, (Dr, wr, Dr))
    g = AD.wgrad(DT.from_numpy(a), DT.from_numpy(L), DT.from_numpy(b), DT.from_numpy(R)).numpy()
    assert rel(g, TA.wgrad(a, L, b, R)) < 1e-12
    s = AD._swap13(DT.from_numpy(L), conj=True).numpy()
    assert np.array_equal(s, np.conj(np.transpose(L, (2, 1, 0))))


def test_expm_nodes():
    rng = np.random.default_rng(4)
    D, w = 6, 3
    Wt = TA.tfi_site_tensor(1.1).astype(np.complex128)
    Lm = crand(rng, (D, w, D)); Lm = 0.5 * (Lm + np.conj(np.transpose(Lm, (2, 1, 0))))
    Rm = crand(rng, (D, w, D)); Rm = 0.5 * (Rm + np.conj(np.transpose(Rm, (2, 1, 0))))
    x = crand(rng, (D, 2, D))
    op = fm.HeffOp("ac", DT.from_numpy(Lm), DT.from_numpy(Rm), W1=Wt, dtype=np.complex128)
    nodes = np.array([0.1, 0.5, 1.0])
    vecs, err = AD.expm_nodes(op, -0.05j, DT.from_numpy(x), nodes, 30)
    H = TA._heff("ac", Wt, Lm, Rm, x.shape)
    for s, v in zip(nodes, vecs):
        ref = scipy.linalg.expm(s * -0.05j * H) @ x.ravel(order="F")
        assert rel(v.numpy().ravel(order="F"), ref) < 1e-10
    assert err < 1e-10


def _state(L, D, seed):
    rng = np.random.default_rng(seed)
    mps = randommps(L, 2, D, rng, dtype=np.complex128)
    mps, _ = canonicalize(mps, normalize=True)
    h = 1.0 + 0.1 * rng.standard_normal(L)
    return mps, h


def _fd(h, mps, dt, nsteps, site, Z, exptol, idx, step=1e-5):
    out = []
    for i in idx:
        vals = []
        for sgn in (1, -1):
            hh = np.array(h, dtype=float)
            hh[i] += sgn * step
            psi = fm.FiniteMPS([DT.from_numpy(A, dtype=np.complex128) for A in mps])
            env = fm.environments(fm.tfi_mpo(hh), psi)
            alg = fm.TDVP1(stepsize=dt, D=max(A.shape[2] for A in mps), exptol=exptol,
                           krylovdim=30)
            for _ in range(nsteps):
                fm.sweep_(env, alg)
            vals.append(float(np.real(fm.expectation_local(env.mps, site, Z))))
        out.append((vals[0] - vals[1]) / (2 * step))
    return np.array(out)


@pytest.mark.parametrize("L,D,nsteps,checkpoint", [(5, 4, 2, 10), (6, 4, 3, 2)])
def test_tdvp1_gradient(L, D, nsteps, checkpoint):
    mps, h = _state(L, D, 3 + L)
    Z = np.diag([-1.0, 1.0])
    site = 3
    psi = fm.FiniteMPS([DT.from_numpy(A, dtype=np.complex128) for A in mps])
    val, g = AD.tfi_field_gradient(h, psi, -0.05j, nsteps, site, Z, checkpoint=checkpoint,
                                   exptol=1e-12)
    vo, go = TA.loss_and_grad(h, mps, -0.05j, nsteps, site - 1, Z)
    assert abs(val - vo) < 1e-9
    assert rel(g, go) < 1e-6               # against the oracle's plain FP64 adjoint
    gfd = _fd(h, mps, -0.05j, nsteps, site, Z, 1e-12, range(L))
    assert rel(g, gfd) < 1e-6              # against central differences of the device forward


def test_autograd_function_matches_adjoint_and_fd():
    """The torch.autograd.Function boundary (TDVP1Observable through tfi_observable):
    h.grad after loss.backward() equals the direct adjoint and central differences."""
    torch = pytest.importorskip("torch")
    L, D, nsteps, site = 5, 4, 2, 3
    mps, h = _state(L, D, 11)
    Z = np.diag([-1.0, 1.0])
    psi = fm.FiniteMPS([DT.from_numpy(A, dtype=np.complex128) for A in mps])
    ht = torch.tensor(h, dtype=torch.float64, requires_grad=True)
    loss = AD.tfi_observable(ht, psi, -0.05j, nsteps, site, Z, checkpoint=1, exptol=1e-12)
    loss.backward()
    val, g = AD.tfi_field_gradient(h, psi, -0.05j, nsteps, site, Z, checkpoint=1, exptol=1e-12)
    assert abs(loss.item() - val) < 1e-13
    assert rel(ht.grad.numpy(), g) < 1e-12
    gfd = _fd(h, mps, -0.05j, nsteps, site, Z, 1e-12, range(L))
    assert rel(ht.grad.numpy(), gfd) < 1e-6


def test_autograd_function_site_tensor_grads():
    """Gradients with respect to the MPO site tensors themselves (complex leaves)
    are the adjoint's Wbar, in torch's convention dL/dRe W + i dL/dIm W."""
    torch = pytest.importorskip("torch")
    from finitemptools_gb300.utilities import tfi_mpo
    L, D, nsteps, site = 4, 4, 2, 2
    mps, h = _state(L, D, 12)
    Z = np.diag([-1.0, 1.0])
    psi = fm.FiniteMPS([DT.from_numpy(A, dtype=np.complex128) for A in mps])
    Ws = [torch.tensor(np.asarray(W, dtype=np.complex128), requires_grad=True)
          for W in tfi_mpo(h).site_tensors(L)]
    loss = AD.tdvp1_observable(Ws, psi, -0.05j, nsteps, site, Z, checkpoint=10)
    loss.backward()
    _, Wb = AD.tdvp1_gradient(tfi_mpo(h), psi, -0.05j, nsteps, site, Z, checkpoint=10)
    for W, ref in zip(Ws, Wb):
        assert rel(W.grad.numpy(), ref) < 1e-12


def test_tf32x3_gradient_close_to_fp64():
    """The complex 3xTF32 gradient form (exponentials of forward and adjoint on the
    tensor cores, real MPO): within 1e-5 relative of the FP64 adjoint."""
    L, D, nsteps, site = 6, 8, 3, 3
    mps, h = _state(L, D, 13)
    Z = np.diag([-1.0, 1.0])
    psi = fm.FiniteMPS([DT.from_numpy(A, dtype=np.complex128) for A in mps])
    v64, g64 = AD.tfi_field_gradient(h, psi, -0.05j, nsteps, site, Z, checkpoint=2)
    v32, g32 = AD.tfi_field_gradient(h, psi, -0.05j, nsteps, site, Z, checkpoint=2,
                                     precision="tf32x3")
    assert abs(v32 - v64) < 1e-6
    assert rel(g32, g64) < 1e-5
