"""The recompute's complex GEMMs (the zgemm calls of cal_g_and_det_T0,
get_g_scratch_T0 and qdr, src/mod_evolution.f90 / src/mod_matrix.f90) on
both engines against numpy's FP64 product: the compensated double-float
product on the FP32 pipe (engine 0) and the Ozaki-split BF16 product on the
tensor cores (engine 1).

Both are double-float class: the error of an entry is bounded by a small
multiple of 2^-48 times the row-by-column magnitudes.  The tests check
  max |C - C_ref| / (max_k |op(A)(i,k)| max_k |op(B)(k,j)| K) <= 2^-44
entry by entry (K the inner dimension), which holds with room for both, and
exact results where the products and sums are exact in both (small
integers)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2.0 ** -44


def _op(x, t):
    return x.conj().transpose(0, 2, 1) if t == "C" else x


def _rand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _check(ta, tb, a, b, engine):
    from pqmc_allinone_gb300.engine import recompute_gemm_check
    c = recompute_gemm_check(ta, tb, a, b, engine)
    oa, ob = _op(a, ta), _op(b, tb)
    ref = oa @ ob
    k = oa.shape[2]
    scale = (np.abs(oa).max(axis=2)[:, :, None] * np.abs(ob).max(axis=1)[:, None, :]) * k
    err = np.abs(c - ref) / np.maximum(scale, 1e-300)
    return c, ref, float(err.max())


SHAPES = [
    # (m, n, k): the 14x14 recompute's shapes (Ns 392, nelec 196), the 8x8 ones, ragged edges
    (196, 196, 392), (392, 196, 196), (392, 392, 196), (64, 64, 128), (37, 70, 130), (1, 1, 1), (129, 65, 63),
]


@pytest.mark.parametrize("engine", [0, 1])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("N", "C"), ("C", "C")])
@pytest.mark.parametrize("m,n,k", SHAPES)
def test_gemm_matches_fp64(engine, ta, tb, m, n, k):
    rng = np.random.default_rng(m * 1000003 + n * 1009 + k)
    count = 3
    a = _rand(rng, (count, k, m) if ta == "C" else (count, m, k))
    b = _rand(rng, (count, n, k) if tb == "C" else (count, k, n))
    _, _, e = _check(ta, tb, a, b, engine)
    assert e < TOL, e


@pytest.mark.parametrize("engine", [0, 1])
def test_graded_rows_and_columns(engine):
    """Rows of op(A) and columns of op(B) scaled over 2^-30 .. 2^30; the
    Ozaki slices take their grid from each row and column, so the bound
    holds entry by entry.  (Both engines keep FP32's exponent range: the
    double-float form and the tensor-core accumulators.)"""
    rng = np.random.default_rng(7)
    m, n, k = 150, 140, 200
    a = _rand(rng, (2, m, k)) * np.exp2(rng.integers(-30, 31, size=(2, m, 1)))
    b = _rand(rng, (2, k, n)) * np.exp2(rng.integers(-30, 31, size=(2, 1, n)))
    _, _, e = _check("N", "N", a, b, engine)
    assert e < TOL, e


@pytest.mark.parametrize("engine", [0, 1])
def test_zeros_and_small_integers_exact(engine):
    """Small-integer operands: every product and partial sum is exact in
    both engines, so the result is bit-for-bit numpy's; a zero row of op(A)
    and a zero column of op(B) give exact zeros."""
    rng = np.random.default_rng(11)
    m, n, k = 100, 90, 150
    a = rng.integers(-20, 21, size=(2, m, k)) + 1j * rng.integers(-20, 21, size=(2, m, k))
    b = rng.integers(-20, 21, size=(2, k, n)) + 1j * rng.integers(-20, 21, size=(2, k, n))
    a[:, 5, :] = 0
    b[:, :, 7] = 0
    c, ref, _ = _check("N", "N", a, b, engine)
    assert np.array_equal(c, ref)
    assert not np.any(c[:, 5, :]) and not np.any(c[:, :, 7])


def test_orthonormal_gram_accuracy():
    """The Gram matrix of an orthonormalised 392 x 196 string (the CholeskyQR
    input, K = 392 complex): the tensor-core engine within 2e-14 of numpy's
    FP64 product (entries at most 1; its levels 0-4 are exact and summed in
    double-float).  The compensated FP32 product (Dot2) sums its low-order
    parts in one FP32 word whose own rounding grows like K^1.5 u^2: measured
    ~1e-12 here, held to 5e-12."""
    rng = np.random.default_rng(3)
    x, _ = np.linalg.qr(_rand(rng, (392, 196)))
    x = x[None]
    from pqmc_allinone_gb300.engine import recompute_gemm_check
    ref = x.conj().transpose(0, 2, 1) @ x
    e1 = np.abs(recompute_gemm_check("C", "N", x, x, 1) - ref).max()
    e0 = np.abs(recompute_gemm_check("C", "N", x, x, 0) - ref).max()
    print(f"orthonormal Gram: max error engine 1 {e1:.3e}, engine 0 {e0:.3e}")
    assert e1 < 2e-14
    assert e0 < 5e-12


def test_bad_arguments_are_errors():
    from pqmc_allinone_gb300.abi import load_library
    import ctypes
    lib = load_library()
    z = np.zeros(16)
    p = z.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert lib.pqmc_recompute_gemm_check(b"N", b"N", 2, 2, 2, 1, p, 1, p, 2, p, 2, 1) != 0   # lda < m
    assert lib.pqmc_recompute_gemm_check(b"T", b"N", 2, 2, 2, 1, p, 2, p, 2, p, 2, 1) != 0   # op 'T'
    assert lib.pqmc_recompute_gemm_check(b"N", b"N", 2, 2, 2, 1, p, 2, p, 2, p, 2, 2) != 0   # engine
