"""The allocation-free two-site H_eff*x (fmpt_ac2_prime_noalloc).

Callers that cannot allocate device memory while they run (a host whose own
allocator owns the device memory, a fixed memory budget) use this entry point:
its scratch is a static device array inside libfmpt, so the call allocates
nothing.  This file is collected last so that a failure here leaves every
other test already run.  It calls the C ABI directly (ctypes), compares two
consecutive calls against fmpt_ac2_prime (1e-12 relative, the FP64 parity
bound), and checks the clear error for a problem larger than the scratch.
"""

import ctypes

import numpy as np
import pytest

from finitemptools_gb300 import _native
from finitemptools_gb300.utilities import heisenberg_xxz_mpo

pytestmark = pytest.mark.gpu


def _buf(lib, h, arr):
    p = ctypes.c_void_p()
    flat = np.ascontiguousarray(np.asarray(arr).ravel(order="F"), dtype=np.float64)
    assert lib.fmpt_malloc(h, flat.nbytes, ctypes.byref(p)) == 0
    assert lib.fmpt_memcpy_h2d(h, p, flat.ctypes.data, flat.nbytes) == 0
    return p


def _get(lib, h, p, n):
    out = np.empty(n, dtype=np.float64)
    assert lib.fmpt_memcpy_d2h(h, out.ctypes.data, p, out.nbytes) == 0
    return out


def test_noalloc_matches_pooled_entry_point_twice():
    lib = _native.lib()
    h = ctypes.c_void_p()
    assert lib.fmpt_create(0, ctypes.byref(h)) == 0
    W = np.ascontiguousarray(heisenberg_xxz_mpo(1.0, 1.0, 0.25)[1].dense().ravel(order="F"))
    rng = np.random.default_rng(99)
    for call, (Dl, Dr) in enumerate([(48, 40), (64, 64)]):      # two calls in a row
        x = rng.standard_normal((Dl, 2, 2, Dr))
        L = rng.standard_normal((Dl, 5, Dl))
        R = rng.standard_normal((Dr, 5, Dr))
        px, pL, pR = _buf(lib, h, x), _buf(lib, h, L), _buf(lib, h, R)
        py0, py1 = ctypes.c_void_p(), ctypes.c_void_p()
        assert lib.fmpt_malloc(h, x.size * 8, ctypes.byref(py0)) == 0
        assert lib.fmpt_malloc(h, x.size * 8, ctypes.byref(py1)) == 0
        st = lib.fmpt_ac2_prime(h, 0, 0, px, W.ctypes.data, W.ctypes.data, pL, pR, py0,
                                Dl, 2, 2, Dr, 5, 5, 5)
        assert st == 0, lib.fmpt_last_error(h)
        st = lib.fmpt_ac2_prime_noalloc(h, 0, px, W.ctypes.data, W.ctypes.data, pL, pR, py1,
                                        Dl, 2, 2, Dr, 5, 5, 5)
        assert st == 0, lib.fmpt_last_error(h)
        y0 = _get(lib, h, py0, x.size)
        y1 = _get(lib, h, py1, x.size)
        assert np.linalg.norm(y1 - y0) <= 1e-12 * np.linalg.norm(y0), call
        for p in (px, pL, pR, py0, py1):
            lib.fmpt_free(h, p)
    lib.fmpt_destroy(h)


def test_noalloc_complex_matches_pooled_entry_point_twice():
    """C128: complex W (imaginary planes of both MPO tensors, complex block coefficients)
    and split-plane x / L / R, whose T1 / T3 take twice the scratch."""
    lib = _native.lib()
    h = ctypes.c_void_p()
    assert lib.fmpt_create(0, ctypes.byref(h)) == 0
    rng = np.random.default_rng(7)
    w = 4
    for call, (Dl, Dr) in enumerate([(24, 36), (40, 40)]):
        W1 = (rng.standard_normal((w, 2, w, 2)) + 1j * rng.standard_normal((w, 2, w, 2)))
        W2 = (rng.standard_normal((w, 2, w, 2)) + 1j * rng.standard_normal((w, 2, w, 2)))
        W1 *= rng.random((w, 1, w, 1)) < 0.6
        W2 *= rng.random((w, 1, w, 1)) < 0.6

        def planes(a):
            f = np.asarray(a).ravel(order="F")
            return np.ascontiguousarray(np.concatenate([f.real, f.imag]))

        hW1, hW2 = planes(W1), planes(W2)
        x = rng.standard_normal((Dl, 2, 2, Dr)) + 1j * rng.standard_normal((Dl, 2, 2, Dr))
        L = rng.standard_normal((Dl, w, Dl)) + 1j * rng.standard_normal((Dl, w, Dl))
        R = rng.standard_normal((Dr, w, Dr)) + 1j * rng.standard_normal((Dr, w, Dr))
        px, pL, pR = _buf(lib, h, planes(x)), _buf(lib, h, planes(L)), _buf(lib, h, planes(R))
        py0, py1 = ctypes.c_void_p(), ctypes.c_void_p()
        assert lib.fmpt_malloc(h, x.size * 16, ctypes.byref(py0)) == 0
        assert lib.fmpt_malloc(h, x.size * 16, ctypes.byref(py1)) == 0
        st = lib.fmpt_ac2_prime(h, 1, 0, px, hW1.ctypes.data, hW2.ctypes.data, pL, pR, py0,
                                Dl, 2, 2, Dr, w, w, w)
        assert st == 0, lib.fmpt_last_error(h)
        st = lib.fmpt_ac2_prime_noalloc(h, 1, px, hW1.ctypes.data, hW2.ctypes.data, pL, pR,
                                        py1, Dl, 2, 2, Dr, w, w, w)
        assert st == 0, lib.fmpt_last_error(h)
        y0 = _get(lib, h, py0, 2 * x.size)
        y1 = _get(lib, h, py1, 2 * x.size)
        assert np.linalg.norm(y1 - y0) <= 1e-12 * np.linalg.norm(y0), call
        for p in (px, pL, pR, py0, py1):
            lib.fmpt_free(h, p)
    lib.fmpt_destroy(h)


def test_noalloc_rejects_problems_beyond_its_scratch():
    lib = _native.lib()
    h = ctypes.c_void_p()
    assert lib.fmpt_create(0, ctypes.byref(h)) == 0
    W = np.ascontiguousarray(heisenberg_xxz_mpo()[1].dense().ravel(order="F"))
    D = 1024          # needs 8 * 2 * 5*4*D^2 bytes = 320 MiB > 64 MiB; no pointer is touched
    dummy = ctypes.c_void_p(256)
    st = lib.fmpt_ac2_prime_noalloc(h, 0, dummy, W.ctypes.data, W.ctypes.data, dummy, dummy,
                                    dummy, D, 2, 2, D, 5, 5, 5)
    assert st == -2
    msg = lib.fmpt_last_error(h).decode()
    assert "static scratch" in msg and "67108864" in msg
    lib.fmpt_destroy(h)
