"""Host logic of the gradient boundary (no GPU): the torch-built TFI site tensors
equal utilities.tfi_mpo's, and autograd through them gives the same field gradient
as the adjoint's own reduction of the site-tensor cotangents."""

import numpy as np
import pytest

from finitemptools_gb300 import adjoint as AD
from finitemptools_gb300.utilities import tfi_mpo


def test_tfi_mpo_torch_matches_host_mpo():
    torch = pytest.importorskip("torch")
    h = np.array([0.3, 1.1, -0.7, 2.0])
    Ws = AD.tfi_mpo_torch(torch.tensor(h))
    for W, ref in zip(Ws, tfi_mpo(h).site_tensors(len(h))):
        assert np.array_equal(W.numpy(), np.asarray(ref, dtype=np.complex128))


def test_field_chain_rule_matches_adjoint_reduction():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    h = rng.standard_normal(5)
    Wb = [rng.standard_normal((3, 2, 3, 2)) + 1j * rng.standard_normal((3, 2, 3, 2))
          for _ in h]
    ht = torch.tensor(h, requires_grad=True)
    Ws = AD.tfi_mpo_torch(ht)
    # a loss whose torch gradient with respect to W_i is exactly Wb_i
    loss = sum(torch.sum(torch.conj(torch.from_numpy(g)) * W).real for g, W in zip(Wb, Ws))
    loss.backward()
    assert np.allclose(ht.grad.numpy(), AD._field_grad(Wb), rtol=1e-14, atol=1e-14)


def test_checkpoint_must_be_positive():
    with pytest.raises(ValueError):
        AD.tdvp1_forward(tfi_mpo([1.0, 1.0]), [None, None], -0.05j, 1, 1, np.eye(2),
                         checkpoint=0)
