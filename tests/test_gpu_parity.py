"""GPU vs oracle parity through the C-ABI (the reference's subroutine order).

Bars: G within 1e-10 relative Frobenius of the FP64 oracle; field, accept
counters and ran2 state bit-identical (which pins the accept/reject sequence);
weights within 1e-9 relative.
"""
import numpy as np
import pytest

from tests.helpers import SEED_WORDS, epsoc_model, epsocz_small, general_bond_model, rel_fro

pytestmark = pytest.mark.gpu

G_TOL = 1e-10


@pytest.fixture(scope="module")
def engine():
    from pqmc_allinone_gb300 import engine
    return engine


def _pair(builder, **kw):
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f = builder(**kw)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS)
    g = PqmcChain(m, field=f, rng_words=SEED_WORDS)
    return m, o, g


MODELS = [
    ("epsocz", epsocz_small, {}),
    ("epsocz_soc", epsocz_small, {"alpha": 0.3, "bc": (1.0, 1.0)}),
    ("epsoc", epsoc_model, {}),
    ("general", general_bond_model, {}),
]


@pytest.mark.parametrize("name,builder,kw", MODELS, ids=[m[0] for m in MODELS])
def test_init_g(engine, name, builder, kw):
    m, o, g = _pair(builder, **kw)
    o.init_expkv(); g.init_expkv()
    o.init_g(1); g.init_g(1)
    assert rel_fro(g.g(), o.g()) < G_TOL
    so, sg = o.state(), g.state()
    assert abs(sg["ln_cw"].real - so["ln_cw"].real) <= 1e-9 * abs(so["ln_cw"].real) + 1e-9
    for blk in range(1, m.nblock + 1):
        qo, do_ = o.qd(blk)
        qg, dg = g.qd(blk)
        assert rel_fro(qg, qo) < 1e-10, blk
        assert np.allclose(dg, do_, rtol=1e-10, atol=1e-12), blk


@pytest.mark.parametrize("left", [True, False])
def test_wrap_two_way(engine, left):
    m, o, g = _pair(epsocz_small, alpha=0.3, bc=(1.0, 1.0))
    o.init_expkv(); g.init_expkv()
    rng = np.random.default_rng(3)
    G0 = rng.normal(size=(m.ns, m.ns)) + 1j * rng.normal(size=(m.ns, m.ns))
    o.set_g(G0); g.set_g(G0)
    for pf in range(1, 5):
        if left:
            o.left_evolve_g(7, pf); g.left_evolve_g(7, pf)
        else:
            o.right_evolve_g(7, pf); g.right_evolve_g(7, pf)
    assert rel_fro(g.g(), o.g()) < 1e-13


def test_one_way(engine):
    m, o, g = _pair(general_bond_model)
    o.init_expkv(); g.init_expkv()
    rng = np.random.default_rng(4)
    X = rng.normal(size=(m.ns, 5)) + 1j * rng.normal(size=(m.ns, 5))
    Y = rng.normal(size=(5, m.ns)) + 1j * rng.normal(size=(5, m.ns))
    assert rel_fro(g.left_evolve(3, 2, X), o.left_evolve(3, 2, X)) < 1e-13
    assert rel_fro(g.right_evolve(3, 2, Y), o.right_evolve(3, 2, Y)) < 1e-13


@pytest.mark.parametrize("name,builder,kw", MODELS, ids=[m[0] for m in MODELS])
def test_update_family(engine, name, builder, kw):
    m, o, g = _pair(builder, **kw)
    for c in (o, g):
        c.init_expkv(); c.init_g(1)
    for pf in range(len(m.pf), 0, -1):
        o.right_evolve_g(m.ntime, pf); g.right_evolve_g(m.ntime, pf)
        o.update_phonon_field(pf, m.ntime); g.update_phonon_field(pf, m.ntime)
        so, sg = o.state(), g.state()
        assert sg["rng"] == so["rng"]
        assert (sg["positive_accept"], sg["negative_accept"]) == (so["positive_accept"], so["negative_accept"])
        assert np.array_equal(g.field(), o.field())
        assert rel_fro(g.g(), o.g()) < G_TOL
        assert abs(sg["ln_cw"].real - so["ln_cw"].real) <= 1e-9 * abs(so["ln_cw"].real) + 1e-9


def test_scratch_and_weight(engine):
    m, o, g = _pair(epsocz_small)
    for c in (o, g):
        c.init_expkv(); c.init_g(1)
    for tc in range(1, 11):
        t = m.ntime - tc + 1
        for pf in range(4, 0, -1):
            for c in (o, g):
                c.right_evolve_g(t, pf); c.update_phonon_field(pf, t)
    eo = o.get_g_scratch(m.ntime - 9, False)
    eg = g.get_g_scratch(m.ntime - 9, False)
    assert rel_fro(g.g(), o.g()) < G_TOL
    assert eg[0] < 1e-8 and eo[0] < 1e-8
    wo, wg = o.cal_new_weight(), g.cal_new_weight()
    assert abs(wg.real - wo.real) <= 1e-9 * abs(wo.real)


def test_sweeps_bit_identical(engine):
    """20 sweeps from the same seed: identical accept/reject sequence."""
    m, o, g = _pair(epsocz_small, ntime=40)
    for c in (o, g):
        c.init_expkv(); c.init_g(1)
    for loop in range(1, 21):
        o.sweep(loop, 1); g.sweep(loop, 1)
        so, sg = o.state(), g.state()
        assert sg["rng"] == so["rng"], loop
        assert (sg["positive_accept"], sg["negative_accept"]) == (so["positive_accept"], so["negative_accept"]), loop
        assert np.array_equal(g.field(), o.field()), loop
        assert rel_fro(g.g(), o.g()) < G_TOL, loop


def test_measurement(engine):
    m, o, g = _pair(epsocz_small, bc=(1.0, 1.0))
    for c in (o, g):
        c.init_expkv(); c.init_g(1)
    ro = o.sweep(1, 2, warmup=0, meas_number=1, cap=4)
    rg = g.sweep(1, 2, warmup=0, meas_number=1, cap=4)
    assert ro.shape == rg.shape and ro.shape[0] == 2
    assert np.allclose(rg, ro, rtol=1e-10, atol=1e-12)
