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
