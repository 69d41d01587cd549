"""The C-ABI library builds, loads and exports every declared symbol; with
no GPU it refuses to run (no CPU fallback)."""
import ctypes
import os

import numpy as np
import pytest

from pqmc_allinone_gb300 import abi
from pqmc_allinone_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pqmc_gb300.h")


@pytest.fixture(scope="module")
def lib():
    build()
    return abi.load_library()


def test_exports_every_declared_symbol(lib):
    names = abi.exported_symbols_from_header(HEADER)
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_error_strings(lib):
    assert b"sm_103a" in lib.pqmc_version()
    assert lib.pqmc_kernel_launches() >= 0


def test_null_arguments_are_rejected(lib):
    assert lib.pqmc_create(None, None) != 0
    assert lib.pqmc_get_state(None, None) != 0
    assert lib.pqmc_sweep(None, 1, 1, 0, 1, 0, None, 0, None) != 0


def test_batch_tuning_and_check_entries_validate_before_the_gpu(lib):
    """The tuning setters, the GEMM-engine selector and the validation
    entries reject bad arguments before any CUDA call (so this runs without
    a GPU), with a message naming the rule."""
    i = ctypes.c_int(0)
    assert lib.pqmc_batch_set_flush_tile(None, 64) != 0
    assert lib.pqmc_batch_set_scan_chunk(None, 4) != 0
    assert lib.pqmc_batch_get_scan_chunk(None, ctypes.byref(i), None) != 0
    assert lib.pqmc_batch_set_gemm_engine(None, 1) != 0
    assert lib.pqmc_batch_get_gemm_engine(None, ctypes.byref(i)) != 0
    z = np.zeros(64)
    p = z.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    # op 'T' is not an operation of the recompute; lda below the rows of A; engine 2
    assert lib.pqmc_recompute_gemm_check(b"T", b"N", 2, 2, 2, 1, p, 2, p, 2, p, 2, 1) != 0
    assert b"ta, tb" in lib.pqmc_last_error()
    assert lib.pqmc_recompute_gemm_check(b"N", b"N", 4, 2, 2, 1, p, 2, p, 2, p, 4, 1) != 0
    assert lib.pqmc_recompute_gemm_check(b"N", b"N", 2, 2, 2, 1, p, 2, p, 2, p, 2, 2) != 0
    # the exact round update's check: flush settings 64, 32, 2, 1 only
    s = np.zeros(4, dtype=np.int32)
    assert lib.pqmc_exact_update_check_tile(8, 4, 4, s.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), p, p, 16) != 0
    assert b"flush tile 64, 32, 2 or 1" in lib.pqmc_last_error()


@pytest.mark.skipif(__import__("tests.conftest", fromlist=["has_gpu"]).has_gpu(), reason="GPU present")
def test_no_cpu_fallback():
    from pqmc_allinone_gb300.engine import PqmcChain, PqmcError
    from tests.helpers import SEED_WORDS, epsocz_small
    m, f = epsocz_small()
    with pytest.raises(PqmcError):
        PqmcChain(m, field=f, rng_words=SEED_WORDS)


def test_struct_layout_matches_header():
    # pqmc_model: 16 int32 + 5 double + 12 pointers
    assert ctypes.sizeof(abi.PqmcModel) == 16 * 4 + 5 * 8 + 12 * 8
    assert ctypes.sizeof(abi.PqmcState) == 16 + 8 + 8 + 8 + 8 + 20 + 4 + 8 + 8
    assert abi.N_FIELD == 25 and abi.N_SCALAR == 3
