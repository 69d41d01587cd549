"""Batched chains on the GPU: the FP64 batch reproduces single chains
exactly; the mixed-precision batch stays within its stated error of the
FP64 oracle.  The mixed batch decides its moves from FP32 ratios and, by
default, applies each scan round as an exact Woodbury update of a
double-float G (double-float Gauss-Jordan, Ozaki-split BF16 tensor-core
products, double-float wraps, double-float recompute): G within 1e-8 of the
oracle throughout.  Flush modes 1 and 0 (the scan's FP32 panels folded in
by tcgen05 or mma.sync split-BF16 products, FP32 wrap corrections) keep
their looser bounds."""
import numpy as np
import pytest

from pqmc_allinone_gb300 import model as M
from pqmc_allinone_gb300.rng import seed_words
from tests.helpers import epsocz_small, rel_fro

pytestmark = pytest.mark.gpu

MIXED_G_TOL = 1e-8     # relative Frobenius, G of the mixed form vs the FP64 oracle


def _models(n, L=4, ntime=20):
    out = []
    for i in range(n):
        m, f = epsocz_small(L=L, ntime=ntime, ngroup=10, lam=0.8, alpha=0.3, seed=10 + i)
        out.append((m, f, seed_words(100 + i)))
    return out


def test_fp64_batch_matches_single_chains():
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = _models(3)
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=0)
    b.init()
    b.sweep(1)
    for (m, f, w), ch in zip(ms, b.chains):
        o = OracleChain(m, field=f, seed_words=w, meas=False)
        o.init_expkv(); o.init_g(1); o.sweep(1, 1)
        assert np.array_equal(ch.field(), o.field())
        assert rel_fro(ch.g(), o.g()) < 1e-10


def test_mixed_batch_close_to_oracle():
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = _models(4, L=4, ntime=20)
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.init()
    orc = []
    for (m, f, w) in ms:
        o = OracleChain(m, field=f, seed_words=w, meas=False)
        o.init_expkv(); o.init_g(1)
        orc.append(o)
    b.sweep(1)
    same = 0
    for o, ch in zip(orc, b.chains):
        o.sweep(1, 1)
        if np.array_equal(ch.field(), o.field()):
            same += 1
            assert rel_fro(ch.g(), o.g()) < MIXED_G_TOL
        s1, s2 = ch.state(), o.state()
        assert abs(s1["positive_accept"] - s2["positive_accept"]) <= 2
    assert same >= 3


# Drift of the fast path between two recomputes, as
# ||G_fast - G_scratch||_F / ||G_scratch||_F: with the exact round update
# (mode 2) at most 1e-8 (the target); with the scan's FP32 panels and FP32
# wrap corrections (mode 1) measured 1e-5..1.5e-5 at 8x8 and 14x14 (ngroup=10,
# delay depth 32..128).
MIXED_DRIFT_TOL = {2: 1e-8, 1: 5e-5}
# The recompute itself (double-float CholeskyQR2 + Gauss-Jordan) against the
# FP64 oracle on the same phonon field.
MIXED_RECOMPUTE_TOL = 1e-10


@pytest.mark.parametrize("mode", [2, 1])
def test_mixed_batch_drift_and_recompute_8x8(mode):
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(4):
        m, f = epsocz_small(L=8, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=40 + i)
        ms.append((m, f, seed_words(400 + i)))
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.set_flush(mode)
    b.init()
    for loop in (1, 2):
        b.sweep(loop)
    for (m, _, w), ch in zip(ms, b.chains):
        s = ch.state()
        assert 0.0 < s["err_g_rel_max"] < MIXED_DRIFT_TOL[mode], s
        assert s["positive_accept"] > 0 and s["negative_accept"] > 0
        # the G a sweep ends with is the recompute at the boundary slice: compare
        # with the FP64 oracle on the chain's own (mixed-path) field
        o = OracleChain(m, field=ch.field(), seed_words=w, meas=False)
        o.init_expkv()
        o.init_g(1)
        assert rel_fro(ch.g(), o.g()) < MIXED_RECOMPUTE_TOL


@pytest.mark.parametrize("engine", [1, 0])
@pytest.mark.parametrize("L", [8, 14])
def test_recompute_gemm_engines_match_oracle(L, engine):
    """The recompute's GEMMs on either engine (1: Ozaki-split BF16 on the
    tensor cores, the default; 0: compensated double-float on the FP32 pipe):
    the fast-path drift and the recompute against the FP64 oracle within the
    mixed batch's bounds; at 14x14 the products have the benchmark's shapes
    (Ns 392, nelec 196)."""
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(2):
        m, f = epsocz_small(L=L, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=60 + i)
        ms.append((m, f, seed_words(600 + i)))
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    assert b.gemm_engine() == 1
    b.set_gemm_engine(engine)
    assert b.gemm_engine() == engine
    b.init()
    for (m, _, w), ch in zip(ms, b.chains):
        o = OracleChain(m, field=ch.field(), seed_words=w, meas=False)
        o.init_expkv()
        o.init_g(1)
        assert rel_fro(ch.g(), o.g()) < MIXED_RECOMPUTE_TOL
    for loop in (1, 2):
        b.sweep(loop)
    for (m, _, w), ch in zip(ms, b.chains):
        s = ch.state()
        assert 0.0 < s["err_g_rel_max"] < MIXED_DRIFT_TOL[2], s
        o = OracleChain(m, field=ch.field(), seed_words=w, meas=False)
        o.init_expkv()
        o.init_g(1)
        assert rel_fro(ch.g(), o.g()) < MIXED_RECOMPUTE_TOL


@pytest.mark.parametrize("L", [8, 14])
def test_tcgen05_flush_matches_mma_sync(L):
    """The two rank-K flush engines (tcgen05 with the accumulator in tensor
    memory, and mma.sync split-BF16 tiles) on identical chains: the same
    accept/reject decisions and G equal to FP32 accumulation rounding, over
    slices that end before the stabilised recompute (which would replace G)."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(2):
        m, f = epsocz_small(L=L, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=60 + i)
        ms.append((m, f, seed_words(600 + i)))
    out = []
    for mode in (0, 1):
        b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
        b.set_flush(mode)
        b.init()
        b.sweep_slices(1, 1, 5)
        out.append([(c.field(), c.g(), c.state()) for c in b.chains])
        b.close()
    for (f0, g0, s0), (f1, g1, s1) in zip(*out):
        assert np.array_equal(f0, f1)
        assert s0["positive_accept"] == s1["positive_accept"] and s0["positive_accept"] > 0
        assert rel_fro(g1, g0) < 2e-6


def test_chain_groups_are_independent():
    """A mixed batch of 16 chains runs as two groups on two streams; every
    chain must come out bit-identical to the same chain advanced in a batch
    of 8 (one group): chains share no data."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(16):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=80 + i)
        ms.append((m, f, seed_words(800 + i)))
    res = {}
    for n in (16, 8):
        b = PqmcBatch([m for m, _, _ in ms[:n]], [f for _, f, _ in ms[:n]], [w for _, _, w in ms[:n]], precision=1)
        b.init()
        b.sweep(1)
        res[n] = [(c.field(), c.g(), c.state()["ln_cw"]) for c in b.chains]
        b.close()
    for k in range(8):
        f16, g16, l16 = res[16][k]
        f8, g8, l8 = res[8][k]
        assert np.array_equal(f16, f8) and np.array_equal(g16, g8) and l16 == l8


def test_mixed_observables_within_error_bars():
    """Equal-time observables (ms_take_measurement, every sweep after a
    warm-up) of the batched mixed-precision form agree with the plain FP64
    form within statistical error bars: 32 chains each, the same seeds, means
    compared component by component with the chain-to-chain standard error."""
    from pqmc_allinone_gb300.engine import PqmcBatch, PqmcChain
    C, sweeps, warm = 32, 24, 4
    ms = []
    for i in range(C):
        m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=900 + i)
        ms.append((m, f, seed_words(9000 + i)))
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1, meas=True)
    b.set_measure(warm, 1, 0)
    b.init()
    for loop in range(1, sweeps + 1):
        b.sweep(loop)
    mixed = np.array([b.records(i).mean(axis=0) for i in range(C)])
    assert all(len(b.records(i)) == 0 for i in range(C))   # taken
    b.close()
    plain = []
    for (m, f, w) in ms:
        ch = PqmcChain(m, field=f, rng_words=w, meas=True)
        ch.init_expkv()
        ch.init_g(1)
        rec = ch.sweep(1, sweeps, warmup=warm, meas_interval=1, meas_number=0, cap=sweeps)
        plain.append(rec.mean(axis=0))
        ch.close()
    plain = np.array(plain)
    assert mixed.shape == plain.shape and mixed.shape[0] == C
    for part in (np.real, np.imag):
        a, p = part(mixed), part(plain)
        se = np.sqrt(a.var(axis=0, ddof=1) / C + p.var(axis=0, ddof=1) / C)
        ok = se > 1e-12 * (1 + np.abs(p.mean(axis=0)))
        z = np.abs(a.mean(axis=0) - p.mean(axis=0))[ok] / se[ok]
        assert z.size > 0 and z.max() < 5.0, z.max()
        # components without spread must agree outright
        assert np.allclose(a.mean(axis=0)[~ok], p.mean(axis=0)[~ok], rtol=1e-6, atol=1e-9)


def _run_batch(ms, loops, graphs=False, chains_only=None):
    from pqmc_allinone_gb300.engine import PqmcBatch
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.set_graphs(graphs)
    b.init()
    for loop in loops:
        b.sweep(loop)
    out = [(c.field(), c.g(), c.state()) for c in b.chains]
    n_graphs = b.graph_count()
    classes = b.classes()
    b.close()
    return out, n_graphs, classes


def test_slice_graphs_bit_identical():
    """The family steps of a slice replayed from captured CUDA graphs give
    the same chains, bit for bit, as the same launches issued one by one:
    one graph per direction and G-buffer parity serves every slice."""
    ms = []
    for i in range(3):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=120 + i)
        ms.append((m, f, seed_words(1200 + i)))
    eager, n0, _ = _run_batch(ms, (1, 2), graphs=False)
    graph, n1, _ = _run_batch(ms, (1, 2), graphs=True)
    assert n0 == 0 and n1 == 4      # {backward, forward} x {parity 0, 1}
    for (f0, g0, s0), (f1, g1, s1) in zip(eager, graph):
        assert np.array_equal(f0, f1) and np.array_equal(g0, g1)
        assert s0["ln_cw"] == s1["ln_cw"] and s0["positive_accept"] == s1["positive_accept"]
        assert s0["positive_accept"] > 0


def test_wrap_column_staging_bit_identical(monkeypatch):
    """The wrap with whole columns of G staged in shared memory (bulk copies
    in and out, blocks updated in place) and the gather form that reads and
    writes each block of a cover-item pair directly compute every entry with
    the same arithmetic: the chains come out bit for bit the same."""
    ms = []
    for i in range(3):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=140 + i)
        ms.append((m, f, seed_words(1400 + i)))
    monkeypatch.setenv("PQMC_WRAP_COLS", "0")
    gather, _, _ = _run_batch(ms, (1, 2), graphs=True)
    monkeypatch.setenv("PQMC_WRAP_COLS", "1")
    staged, _, _ = _run_batch(ms, (1, 2), graphs=True)
    for (f0, g0, s0), (f1, g1, s1) in zip(gather, staged):
        assert np.array_equal(f0, f1) and np.array_equal(g0, g1)
        assert s0["ln_cw"] == s1["ln_cw"] and s0["positive_accept"] == s1["positive_accept"]
        assert s0["positive_accept"] > 0


def test_wrap_tiles_bit_identical_and_autotuned():
    """Every tile shape of the wrap (gathered blocks, 1 or 2 column items per
    staged CTA) gives the same chains bit for bit, graphs included; the tile
    autotuner times each, keeps the fastest and the run continues from it."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(3):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=150 + i)
        ms.append((m, f, seed_words(1500 + i)))
    runs = []
    for ci in (0, 1, 2):
        b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
        b.set_wrap_tile(ci)
        assert b.wrap_tile() == ci
        b.init()
        for loop in (1, 2):
            b.sweep(loop)
        runs.append([(c.field(), c.g(), c.state()) for c in b.chains])
        b.close()
    for other in runs[1:]:
        for (f0, g0, s0), (f1, g1, s1) in zip(runs[0], other):
            assert np.array_equal(f0, f1) and np.array_equal(g0, g1)
            assert s0["ln_cw"] == s1["ln_cw"] and s0["positive_accept"] == s1["positive_accept"]
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.init()
    (best, fbest, qbest), table, ftable, qtable = b.autotune_tiles(1, 1, 2)
    assert best in (0, 1, 2) and b.wrap_tile() == best
    assert fbest in (64, 32, 2, 1) and b.flush_tile() == fbest
    assert b.scan_chunk() == qbest and qbest in [q for q, _ in qtable]
    assert all(v is not None and v > 0 for v in table.values())
    assert all(v is not None and v > 0 for v in ftable.values())
    assert all(v is not None and v > 0 for _, v in qtable)
    assert table[best] == min(table.values()) and ftable[fbest] == min(ftable.values())
    assert min(qtable, key=lambda t: t[1])[0] == qbest
    assert b.tiles_timed(table, ftable, qtable) == 10   # 10 slots of 2 slices: all of sweep 1
    b.sweep(2)
    assert all(0.0 < c.state()["err_g_rel_max"] < 1e-8 for c in b.chains)
    b.close()


def test_scan_chunks_bit_identical():
    """The scan's panel chunk (the largest that fits, 6 or 4 columns per stage) changes only
    how the panels stream through shared memory: the chains are bit-identical
    whichever runs."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(3):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=170 + i)
        ms.append((m, f, seed_words(1700 + i)))
    runs = []
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    qmax = b.scan_chunk(with_max=True)[1]
    b.close()
    assert qmax >= 4
    for qc in sorted({qmax, min(qmax, 6), 4}, reverse=True):
        b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
        b.set_scan_chunk(qc)
        assert b.scan_chunk() == qc
        b.init()
        for loop in (1, 2):
            b.sweep(loop)
        runs.append([(c.field(), c.g(), c.state()) for c in b.chains])
        b.close()
    for other in runs[1:]:
        for (f0, g0, s0), (f1, g1, s1) in zip(runs[0], other):
            assert np.array_equal(f0, f1) and np.array_equal(g0, g1)
            assert s0["ln_cw"] == s1["ln_cw"] and s0["positive_accept"] == s1["positive_accept"]
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    with pytest.raises(RuntimeError, match="shared memory"):
        b.set_scan_chunk(10 ** 6)
    b.close()


def test_flush_tiles_agree():
    """The flushes of the exact round update: 128 x 64 tiles at one CTA per
    SM (k_xgemm<1>), 128 x 32 at two (k_xflush2), and the pipeline
    (k_xflushp, 2 or 1 CTAs per row tile).  The last three sum the rounded
    level of the Ozaki products stage by stage, so their chains are bit for
    bit the same; k_xgemm<1> sums it in another order, so it agrees with them
    to that rounding: the same accept/reject sequence here, G within 1e-12,
    all within the drift bound."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(3):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=160 + i)
        ms.append((m, f, seed_words(1600 + i)))
    runs = []
    for ct in (64, 32, 2, 1):
        b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
        b.set_flush_tile(ct)
        assert b.flush_tile() == ct
        b.init()
        for loop in (1, 2):
            b.sweep(loop)
        runs.append([(c.field(), c.g(), c.state()) for c in b.chains])
        b.close()
    for other in runs[1:]:
        for (f0, g0, s0), (f1, g1, s1) in zip(runs[0], other):
            assert np.array_equal(f0, f1) and s0["positive_accept"] == s1["positive_accept"]
            assert rel_fro(g1, g0) < 1e-12
            assert 0.0 < s1["err_g_rel_max"] < MIXED_DRIFT_TOL[2]
    for other in runs[2:]:   # the pipeline against k_xflush2: bit for bit
        for (f1, g1, s1), (f2, g2, s2) in zip(runs[1], other):
            assert np.array_equal(f1, f2) and np.array_equal(g1, g2)
            assert s1["ln_cw"] == s2["ln_cw"]


def test_launch_priorities_bit_identical(monkeypatch):
    """The family-step kernels launched at the highest stream priority (node
    priorities in the slice graphs) and every kernel at the default priority:
    priorities only change which group's CTAs the GPU dispatches first, never
    the order of a group's own kernels, so two chain groups come out bit for
    bit the same."""
    ms = []
    for i in range(16):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=180 + i)
        ms.append((m, f, seed_words(1800 + i)))
    monkeypatch.setenv("PQMC_PRIORITY", "0")
    plain, _, _ = _run_batch(ms, (1, 2), graphs=True)
    monkeypatch.setenv("PQMC_PRIORITY", "3")
    prio, _, _ = _run_batch(ms, (1, 2), graphs=True)
    for (f0, g0, s0), (f1, g1, s1) in zip(plain, prio):
        assert np.array_equal(f0, f1) and np.array_equal(g0, g1)
        assert s0["ln_cw"] == s1["ln_cw"] and s0["positive_accept"] == s1["positive_accept"]
        assert s0["positive_accept"] > 0


def test_uneven_batch_matches_its_classes():
    """A mixed batch of chains of uneven L and Lt (C3-shaped, scaled down)
    splits into geometry classes that interleave on their own streams; every
    chain must come out bit-identical to the same chain advanced in a batch of
    its class alone, and after the sweeps its G (the stabilised recompute at
    the sweep boundary) must match the FP64 oracle on the chain's own field."""
    from oracle.oracle import OracleChain
    rng = np.random.default_rng(7)
    geo = [(4, 20), (6, 40), (4, 40), (6, 20), (4, 20), (6, 40), (4, 40)]
    ms = []
    for i, (L, nt) in enumerate(geo):
        lam = float(rng.uniform(0.5, 1.0))
        m, f = epsocz_small(L=L, ntime=nt, ngroup=10, lam=lam, alpha=0.3, seed=1000 + i)
        ms.append((m, f, seed_words(1000 + i)))
    mixed, n_graphs, classes = _run_batch(ms, (1, 2), graphs=True)
    assert len(classes) == 4 and sum(c["chains"] for c in classes) == len(geo)
    assert sorted((c["ns"], c["ntime"]) for c in classes) == [(32, 20), (32, 40), (72, 20), (72, 40)]
    assert n_graphs == 4 * 4
    for key in sorted(set(geo)):
        idx = [i for i, g in enumerate(geo) if g == key]
        alone, _, _ = _run_batch([ms[i] for i in idx], (1, 2), graphs=False)
        for i, (f1, g1, s1) in zip(idx, alone):
            f0, g0, s0 = mixed[i]
            assert np.array_equal(f0, f1) and np.array_equal(g0, g1), (key, i)
            assert s0["ln_cw"] == s1["ln_cw"] and s0["positive_accept"] == s1["positive_accept"]
    for (m, _, w), (f, g, s) in zip(ms, mixed):
        assert s["positive_accept"] > 0 and s["negative_accept"] > 0
        assert 0.0 < s["err_g_rel_max"] < MIXED_DRIFT_TOL[2], s   # the exact round update in every class
        o = OracleChain(m, field=f, seed_words=w, meas=False)
        o.init_expkv()
        o.init_g(1)
        assert rel_fro(g, o.g()) < MIXED_RECOMPUTE_TOL


def test_uneven_batch_autotune_then_sweeps():
    """Both autotuners on an uneven batch (every class tunes its own depth
    and wrap tile on genuine slices), then the rest of the sweep from the
    slice the timed candidates reached: the fast path stays within the
    drift bound in every class."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    geo = [(4, 80), (6, 80), (4, 80), (6, 80)]
    ms = []
    for i, (L, nt) in enumerate(geo):
        m, f = epsocz_small(L=L, ntime=nt, ngroup=10, lam=0.8, alpha=0.3, seed=1100 + i)
        ms.append((m, f, seed_words(1100 + i)))
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.init()
    best, table = b.autotune(1, 1, 10, (16, 32, 64, 96))
    assert table[96] < 0 and best in (16, 32, 64)   # 96 columns exceed the exact round update
    tc = 1 + 10 * sum(1 for v in table.values() if v >= 0)
    (tile, ftile, qc), ttable, ftable, qtable = b.autotune_tiles(1, tc, 4)
    tc += 4 * b.tiles_timed(ttable, ftable, qtable)
    assert tc <= 80
    b.sweep_slices(1, tc, 80 - tc + 1)
    b.sweep(2)
    assert all(0.0 < c.state()["err_g_rel_max"] < MIXED_DRIFT_TOL[2] for c in b.chains)
    b.close()


def test_fp64_uneven_batch_matches_oracle():
    """An FP64 batch of chains of uneven L and Lt, driven from worker
    threads: every chain's decisions and field match the oracle, bit for
    bit, after a sweep each."""
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcBatch
    geo = [(4, 20), (6, 40), (4, 40), (6, 20), (4, 20)]
    ms = []
    for i, (L, nt) in enumerate(geo):
        m, f = epsocz_small(L=L, ntime=nt, ngroup=10, lam=0.6 + 0.05 * i, alpha=0.3, seed=1100 + i)
        ms.append((m, f, seed_words(1100 + i)))
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=0)
    b.init()
    b.sweep(1)
    for (m, f, w), ch in zip(ms, b.chains):
        o = OracleChain(m, field=f, seed_words=w, meas=False)
        o.init_expkv(); o.init_g(1); o.sweep(1, 1)
        assert np.array_equal(ch.field(), o.field())
        assert ch.state()["positive_accept"] == o.state()["positive_accept"]
        assert rel_fro(ch.g(), o.g()) < 1e-10
    b.close()


def test_batch_field_slices_and_states():
    """pqmc_batch_field_slices moves one block of every chain's field (host
    blocks chain after chain) both ways; pqmc_batch_states equals the
    per-chain states."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(3):
        m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=300 + i)
        ms.append((m, f, seed_words(3000 + i)))
    m = ms[0][0]
    b = PqmcBatch([x for x, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    rng = np.random.default_rng(5)
    blk = rng.normal(scale=0.5, size=(3, 10, m.n_bf))      # chain after chain, (n_bf, 10) column-major each
    b.field_slices(6, 10, blk, True)
    for i, c in enumerate(b.chains):
        assert np.array_equal(c.field()[:, 5:15], blk[i].T)
    back = np.zeros_like(blk)
    b.field_slices(6, 10, back, False)
    assert np.array_equal(back, blk)
    # the chains then run exactly as a batch set up with those fields
    fields = [c.field() for c in b.chains]
    b.init()
    b.sweep(1)
    b2 = PqmcBatch([x for x, _, _ in ms], fields, [w for _, _, w in ms], precision=1)
    b2.init()
    b2.sweep(1)
    for c1, c2 in zip(b.chains, b2.chains):
        assert np.array_equal(c1.field(), c2.field())
    assert b.states() == [c.state() for c in b.chains]
    b.close()
    b2.close()


def test_phase_timers_and_flush_rounds():
    """The phase timers cover every phase of the family step and the device
    count of flushes with columns is at least one per family step with an
    accepted move (and at most the launched rounds)."""
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(2):
        m, f = epsocz_small(L=6, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=700 + i)
        ms.append((m, f, seed_words(7000 + i)))
    b = PqmcBatch([x for x, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.init()
    b.set_timing(True)
    b.sweep_slices(1, 1, 10)
    ph = b.timing()
    rounds = b.flush_rounds()
    b.set_timing(False)
    assert set(ph) == set(PqmcBatch.PHASES)
    for k in ("prep", "scan", "flush", "wrap", "recompute", "split"):
        assert ph[k][0] > 0 and ph[k][1] > 0, k
    launched = ph["flush"][1]
    assert all(0 < r <= launched for r in rounds), (rounds, launched)
    assert b.flush_rounds() == [0, 0]          # set_timing clears the counts
    b.close()
