"""The Ozaki slicing of the tensor-core products (ozaki.cuh, used by the
exact round update with 5 slices and by the recompute's GEMMs with 6),
restated in numpy float32 and checked against the claims the kernels rest
on:

- piece s of a value on the grid 2^(e - 8(s+1)) is an integer of at most
  256 grid units (129 after the first), so it is exact in BF16 (8
  significant bits);
- the pieces rebuild the double-float value (hi + lo) to within the last
  grid, 2^(e - 8 NS);
- a product of two pieces is exact in FP32, and for an inner dimension of
  128 real terms the sum of one level i + j = l stays below 2^24 grid units
  for l <= 4: levels 0-4 of a chunk are exact FP32 sums, whatever the order
  the tensor core adds them in.

Runs on the CPU only; no GPU, no library call."""
import numpy as np
import pytest

F32 = np.float32


def two_sum(a, b):
    s = F32(a + b)
    bb = F32(s - a)
    e = F32(F32(a - F32(s - bb)) + F32(b - bb))
    return s, e


def oz_exp(vmax, floor):
    """The exponent e with vmax < 2^e (vmax >= 0), at least floor (oz_exp_f)."""
    if vmax <= 0:
        return floor
    b = (np.array(vmax, dtype=np.float32).view(np.int32) >> 23) & 0xFF
    return max(int(b) - 126, floor)


def oz_split(h, l, e, ns):
    """The ns pieces of the double-float value (h, l) for the exponent e (oz_split_n)."""
    q = []
    h, l = F32(h), F32(l)
    for s in range(ns):
        sh = 8 * (s + 1) - e
        v = F32(np.rint(F32(h * F32(2.0) ** sh)))
        qs = F32(v * F32(2.0) ** (-sh))
        q.append(qs)
        h = F32(h - qs)   # exact: h and qs lie within half a grid step
        h, l = two_sum(h, l)
    return q


def df_of(x):
    """double -> (hi, lo) in float32, as df_make."""
    hi = F32(x)
    lo = F32(x - np.float64(hi))
    return hi, lo


def bf16_exact(x):
    """x has at most 8 significant bits (BF16 keeps 8)."""
    if x == 0:
        return True
    m, _ = np.frexp(np.float64(x))
    return float(m * 256) == np.round(m * 256)


@pytest.mark.parametrize("ns,floor", [(5, -80), (6, -78)])
def test_pieces_exact_in_bf16_and_rebuild_the_value(ns, floor):
    rng = np.random.default_rng(ns)
    for scale in (1e-6, 1.0, 3.7e5):
        row = rng.standard_normal(64) * scale * np.exp(rng.uniform(-3, 3, 64))
        dfs = [df_of(x) for x in row]
        e = oz_exp(max(abs(h) for h, _ in dfs), floor)
        for x, (h, l) in zip(row, dfs):
            q = oz_split(h, l, e, ns)
            for s, qs in enumerate(q):
                units = np.float64(qs) * 2.0 ** (8 * (s + 1) - e)
                assert units == np.round(units)
                assert abs(units) <= (256 if s == 0 else 129)
                assert bf16_exact(qs)
            rest = (np.float64(h) + np.float64(l)) - sum(np.float64(v) for v in q)
            assert abs(rest) <= 2.0 ** (e - 8 * ns)


def test_level_sums_below_2_to_24_units_for_128_terms():
    """Worst case and random rows: the level-l sum of a 128-term chunk in
    units of its grid 2^(ea + eb - 8(l + 2)) is an integer below 2^24 for
    l <= 4 (so FP32 holds it exactly), and level 5 can exceed it."""
    def bound(l):
        # pairs (i, l - i): two pairs touch a first piece (<= 256 x 129), the
        # rest are <= 129 x 129; l = 0 is 256 x 256
        if l == 0:
            return 256 * 256
        return 2 * 256 * 129 + (l - 1) * 129 * 129
    for l in range(5):
        assert 128 * bound(l) < 2 ** 24, l
    assert 128 * bound(5) > 2 ** 24
    rng = np.random.default_rng(7)
    ns = 6
    a = rng.standard_normal(128)
    b = rng.standard_normal(128)
    ea = oz_exp(max(abs(F32(x)) for x in a), -78)
    eb = oz_exp(max(abs(F32(x)) for x in b), -78)
    qa = [oz_split(*df_of(x), ea, ns) for x in a]
    qb = [oz_split(*df_of(x), eb, ns) for x in b]
    for l in range(ns):
        units = 0
        for k in range(128):
            for i in range(l + 1):
                j = l - i
                p = np.float64(qa[k][i]) * np.float64(qb[k][j])
                assert F32(p) == p   # the product of two pieces is exact in FP32
                u = p * 2.0 ** (8 * (l + 2) - ea - eb)
                assert u == np.round(u)
                units += int(u)
        if l <= 4:
            assert abs(units) < 2 ** 24
    # the level sums rebuild the product to the last level's grid
    exact = sum(np.float64(x) * np.float64(y) for x, y in zip(a, b))
    rebuilt = 0.0
    for l in range(ns):
        for i in range(l + 1):
            rebuilt += sum(np.float64(qa[k][i]) * np.float64(qb[k][l - i]) for k in range(128))
    assert abs(rebuilt - exact) <= 128 * 2.0 ** (ea + eb - 46)
