"""CPU checks of the C-ABI library and the host-side logic (no GPU needed)."""

import ctypes
import os
import re

import numpy as np
import pytest

import finitemptools_gb300 as fm
from finitemptools_gb300 import _native
from finitemptools_gb300.mps import OneBased, max_bond_dimensions
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "fmpt.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fmpt_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_every_header_symbol():
    from finitemptools_gb300 import build
    build.build()
    lib = ctypes.CDLL(_native.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes table covers exactly the header
    assert sorted(_native.SIGNATURES) == syms


def test_status_strings_and_no_gpu_behaviour():
    lib = _native.lib()
    assert lib.fmpt_version() >= 1
    assert lib.fmpt_status_string(-2) == b"dimension mismatch"
    h = ctypes.c_void_p()
    st = lib.fmpt_create(0, ctypes.byref(h))
    if st != 0:          # no GPU here: a clean error, never a crash
        assert st in (-3, -1)
        with pytest.raises(fm.FMPTError):
            fm.Handle(0)
    else:
        lib.fmpt_destroy(h)


def test_one_based_and_bond_dims_match_oracle():
    ob = OneBased([10, 20, 30])
    assert ob[1] == 10 and ob[3] == 30
    with pytest.raises(IndexError):
        ob[0]
    for L, d, D in [(6, 2, 8), (20, 2, 64), (5, 4, 50), (3, 3, 2)]:
        assert max_bond_dimensions([d] * L, D) == O.max_virtual_dims([d] * L, D)


def test_schur_tensor_checks():
    from finitemptools_gb300.utilities import SchurMPOTensor, spin_half_matrices
    p = spin_half_matrices()
    with pytest.raises(ValueError):
        SchurMPOTensor([[np.eye(2), 0], [p["z"], np.eye(2)]])   # lower triangle
    t = fm.heisenberg_xxz_mpo(1.0, 1.0, 0.0)[1]
    assert t.keys() == [(0, 0), (0, 1), (0, 2), (0, 3), (1, 4), (2, 4), (3, 4), (4, 4)]
    j = fm.j1j2_heisenberg_mpo()[1]
    assert j.isscal(1, 4) and not j.isscal(0, 1)


def test_host_buffers_split_planes():
    from finitemptools_gb300.device import to_host_buffer
    a = np.arange(6).reshape(2, 3) + 1j * np.arange(6).reshape(2, 3)
    b = to_host_buffer(a, np.complex128)
    assert np.allclose(b[:6], a.real.ravel(order="F"))
    assert np.allclose(b[6:], a.imag.ravel(order="F"))
    with pytest.raises(TypeError):
        to_host_buffer(a, np.float64)
