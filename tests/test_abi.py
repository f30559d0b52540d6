"""The C-ABI library loads, exports every symbol include/hmgpu.h declares, and
its host-only entry points behave (no GPU compute is called here)."""
import ctypes
import os
import re

import numpy as np

import hierarchicalmatrices as hm
from hierarchicalmatrices import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "hmgpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hm_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported():
    syms = declared_symbols()
    assert len(syms) >= 15
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(_lib.EXPORTED), sorted(set(syms) ^ set(_lib.EXPORTED))


def test_status_strings():
    for code in range(11):
        assert _lib.lib.hm_status_string(code).decode() != "unknown status"
    assert _lib.lib.hm_status_string(99).decode() == "unknown status"
    assert _lib.lib.hm_version() >= 100


def test_blockrank():
    assert hm.BLOCKRANK(np.float64) == 20
    assert hm.BLOCKRANK(np.float32) == 10
    assert hm.BLOCKSIZE(np.float64) == 80
    assert hm.BLOCKRANK(np.float16) % 2 == 0


def test_kernels_callable():
    x, y = np.array([1.0, 2.0]), np.array([0.5, 0.25])
    np.testing.assert_allclose(hm.cauchykernel(x, y), 1 / (x - y))
    np.testing.assert_allclose(hm.logkernel(x, y), np.log(np.abs(x - y)))
    assert sorted(hm.KERNELS) == ["cauchykernel", "coulombkernel", "coulombprimekernel", "logkernel"]


def test_null_arguments_rejected_without_a_gpu():
    """Argument checks that happen before any CUDA call: NULL handles and
    invalid counts return status codes (no GPU needed)."""
    L = _lib.lib
    assert L.hm_autotune(None, 1, 1, None, None, None) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_configure(None, _lib.HM_OPT_PDL, 1) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_mul(None, None, 0, None, 0, 1, 1, None) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_mul_noalloc(None, None, None, 1, None) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_mul_host(None, None, None, 1, 1) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_profile_timeline(None, None, 0) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_trtri_batched(_lib.HM_F64, -1, None, None) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_potrf_batched_async(_lib.HM_F64, 1, None, None, None) == _lib.HM_ERR_INVALID_ARG
    assert L.hm_solve_transposed(_lib.HM_F64, -1, None, None, 0, 0, None) == _lib.HM_ERR_INVALID_ARG
