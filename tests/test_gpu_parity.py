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


def _c1_model():
    """The 4x4 configuration with phonon-modulated bonds t(1 - lambda x_b),
    lambda = 0.8, 32 bonds, spin 1/2 as ncopy = 2 (weight det^ncopy,
    src/mod_update.f90:104), Nup = Ndn = 8, Lt = 80, dtau = 0.1, ngroup = 10,
    the Gaussian proposal with sigma = 0.3 and x ~ N(0, 0.5^2) from seed 1."""
    import dataclasses
    from pqmc_allinone_gb300 import model as M
    m1, f = general_bond_model(L=4, ntime=80, ngroup=10, lam=0.8, seed=1)
    spec = dataclasses.replace(m1.spec, ncopy=2, proposal_kind=M.PROPOSAL_GAUSSIAN, jump_distance=0.3)
    m = M.build_model(spec, twist_seed=3, twist=1e-3)
    assert m.n_bf == 32 and m.nelec == 8 and m.ntime == 80
    return m, f


def test_spin_half_gaussian_20_sweeps_bit_identical(engine):
    """The spin-1/2 bond-model configuration with the Gaussian proposal: 20
    sweeps from one seed give the oracle's accept/reject sequence bit for bit
    (ran2 state, counters and field after every sweep), G within 1e-10.  The
    Box-Muller jumps use the fixed-order arithmetic both sides share."""
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f = _c1_model()
    o = OracleChain(m, field=f, seed_words=SEED_WORDS)
    g = PqmcChain(m, field=f, rng_words=SEED_WORDS)
    for c in (o, g):
        c.init_expkv()
        c.init_g(1)
    for loop in range(1, 21):
        o.sweep(loop, 1)
        g.sweep(loop, 1)
        so, sg = o.state(), g.state()
        assert sg["rng"] == so["rng"], loop
        assert (sg["positive_accept"], sg["negative_accept"]) == (so["positive_accept"], so["negative_accept"]), loop
        assert np.array_equal(g.field(), o.field()), loop
        assert rel_fro(g.g(), o.g()) < G_TOL, loop
    assert so["positive_accept"] > 0 and so["negative_accept"] > 0


def test_spin_half_gaussian_mixed_batch(engine):
    """The same configuration through the mixed batch (exact round update,
    dim-2 plaquettes, Gaussian proposals formed on the device): the fast
    path stays within 1e-8 of the recompute, and the G a sweep ends with
    matches the oracle's on the chain's own field."""
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcBatch
    from pqmc_allinone_gb300.rng import seed_words
    m, f = _c1_model()
    words = [seed_words(20 + i) for i in range(4)]
    b = PqmcBatch([m] * 4, [f] * 4, words, precision=1)
    b.init()
    for loop in (1, 2):
        b.sweep(loop)
    for ch, w in zip(b.chains, words):
        s = ch.state()
        assert 0.0 < s["err_g_rel_max"] < 1e-8, s
        assert s["positive_accept"] > 0
        o = OracleChain(m, field=ch.field(), seed_words=w, meas=False)
        o.init_expkv()
        o.init_g(1)
        assert rel_fro(ch.g(), o.g()) < 1e-10
    b.close()


def test_c2_full_size_plain_fp64():
    """The production-size configuration (14x14 spin-orbit lattice, Ns = 392,
    Nup = 196, Lt = 1000, dtau = 0.1, lambda = 0.8, static alpha = 0.3,
    ngroup = 10, x ~ N(0, 0.5^2) from seed 2) on the plain FP64 path against
    the oracle: G of init_g_T0 within 1e-10, then one stabilisation block of
    the first sweep (ten slices of updates and wraps closed by the
    recompute, src/Main_PQMC.f90:99-154) with the same accept/reject sequence
    and G within 1e-10 (err_fast, src/mod_evolution.f90:179-193, on both)."""
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300 import model as M
    from pqmc_allinone_gb300.engine import PqmcChain
    spec = M.epsocz_spec(14, lam=0.8, alpha=0.3, ntime=1000, ngroup=10, filling=0.5, jump_distance=0.5)
    m = M.build_model(spec, twist_seed=11, twist=1e-3)
    assert (m.ns, m.nelec, m.ntime, m.n_bf) == (392, 196, 1000, 392)
    f = M.field_gaussian(m, 2)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)
    g = PqmcChain(m, field=f, rng_words=SEED_WORDS)
    for c in (o, g):
        c.init_expkv()
        c.init_g(1)
    assert rel_fro(g.g(), o.g()) < G_TOL
    o.sweep(1, 1, max_slices=m.ngroup)
    g.sweep_slices(1, 1, m.ngroup)
    so, sg = o.state(), g.state()
    assert sg["rng"] == so["rng"]
    assert (sg["positive_accept"], sg["negative_accept"]) == (so["positive_accept"], so["negative_accept"])
    assert sg["positive_accept"] > 1000
    assert np.array_equal(g.field(), o.field())
    assert rel_fro(g.g(), o.g()) < G_TOL
    assert abs(sg["ln_cw"].real - so["ln_cw"].real) <= 1e-9 * abs(so["ln_cw"].real)
