"""The C-ABI library builds, loads on the CPU and exports every entry point of include/efgpu.h."""

import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def _declared():
    txt = open(os.path.join(ROOT, "include", "efgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ef_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from edelweissfe_gb300 import _lib, build

    build.build()
    lib = _lib.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)
    assert lib.ef_abi_version() == 3


def test_argument_validation_without_gpu():
    from edelweissfe_gb300 import _lib

    lib = _lib.load()
    ctx = ctypes.c_void_p()
    X = np.zeros(7)
    assert lib.ef_create(7, X.ctypes.data, ctypes.byref(ctx)) == _lib.EF_ERR_ARG  # not a multiple of 3
    assert b"multiple of 3" in lib.ef_last_error()
    assert lib.ef_create(0, X.ctypes.data, ctypes.byref(ctx)) == _lib.EF_ERR_ARG
    assert lib.ef_finalize(None, 0) == _lib.EF_ERR_ARG
    assert lib.ef_compute_elements(None, None, None, None, 0.0, None, None, None) == _lib.EF_ERR_STATE
    # calls on a missing context fail with EF_ERR_STATE before touching the device
    cid = ctypes.c_int(-1)
    assert lib.ef_results_create(None, 0, None, 0, None, 0, 0, 6, ctypes.byref(cid)) == _lib.EF_ERR_STATE
    assert cid.value == -1
    assert lib.ef_results_update(None, 0, 0, None, None) == _lib.EF_ERR_STATE
    assert lib.ef_results_destroy(None, 0) == _lib.EF_ERR_STATE
    assert lib.ef_reset_state(None) == _lib.EF_ERR_STATE
    assert lib.ef_accept_state(None) == _lib.EF_ERR_STATE
