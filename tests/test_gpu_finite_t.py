"""The finite-temperature path on the GPU (init_g_FT, get_g_scratch_FT,
cal_new_weight_FT, the FT sweep; src/mod_evolution.f90:409-785) against the
CPU restatement oracle/finite_t.py and the known answers it is pinned to.

The GPU strings use a column-pre-pivoted Householder QR; the oracle uses
LAPACK's column-pivoted QR (zgeqp3).  The two decompositions differ, the
products they represent do not, so G and Re ln_cw agree to rounding:
1e-10 relative Frobenius for G, 1e-9 relative for the weight.
"""
import numpy as np
import pytest

from tests.helpers import SEED_WORDS, epsocz_small, general_bond_model, rel_fro

pytestmark = pytest.mark.gpu

G_TOL = 1e-10
W_TOL = 1e-9
# Im ln_cw is reduced modulo 2 pi in single precision, as the reference
# reduces it (mod(aimag, 2*pi), src/mod_evolution.f90:626); two evaluations
# whose phases differ by k whole turns before the reduction differ by
# k (2 pi_sp - 2 pi) = k * 1.75e-7 after it.  The phase check allows 50 turns.
PHASE_TOL = 50 * 1.75e-7 + 1e-9


def _pair(builder, **kw):
    from oracle.finite_t import FiniteT
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f = builder(**kw)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)
    o.init_expkv()
    g = PqmcChain(m, field=f, rng_words=SEED_WORDS)
    g.set_temperature(False)
    g.init_expkv()
    return m, o, FiniteT(o), g


MODELS = [
    ("epsocz", epsocz_small, {"ntime": 20, "ngroup": 5}),
    ("epsocz_soc", epsocz_small, {"ntime": 20, "ngroup": 5, "alpha": 0.3, "bc": (1.0, 1.0)}),
    ("general", general_bond_model, {"ntime": 20, "ngroup": 4}),
]


@pytest.mark.parametrize("name,builder,kw", MODELS, ids=[m[0] for m in MODELS])
def test_init_g_ft_matches_oracle_and_dense(name, builder, kw):
    from oracle.finite_t import dense_g_and_weight
    m, o, ft, g = _pair(builder, **kw)
    assert not g.proj()
    g.init_g(1)                                   # dispatches to init_g_FT
    go, lo = ft.init_g(1)
    gd, ld = dense_g_and_weight(o)
    assert rel_fro(g.g(), go) < G_TOL
    assert rel_fro(g.g(), gd) < G_TOL
    w = g.state()["ln_cw"]
    assert abs(w.real - lo.real) <= W_TOL * abs(lo.real) + 1e-9
    assert abs(np.exp(1j * w.imag) - np.exp(1j * lo.imag)) < PHASE_TOL
    wn = g.cal_new_weight()                       # cal_new_weight_FT
    assert abs(wn.real - lo.real) <= W_TOL * abs(lo.real) + 1e-9
    assert rel_fro(g.g(), go) < G_TOL             # G untouched by the weight


@pytest.mark.parametrize("ntime,ngroup", [(400, 10), (1000, 20)])
def test_free_fermions_long_beta(ntime, ngroup):
    """lambda = 0 at beta = 40 and 100: the GPU strings against the
    eigen-decomposition answer (no stabilised code on the reference side)."""
    from oracle.finite_t import free_fermion_g
    m, o, ft, g = _pair(epsocz_small, L=4, ntime=ntime, ngroup=ngroup, lam=0.0, alpha=0.3)
    g.init_g_ft(1)
    gf, ref = free_fermion_g(o)
    assert rel_fro(g.g(), gf) < 1e-9
    w = g.state()["ln_cw"]
    assert abs(w.real - ref) <= 1e-10 * abs(ref) + 1e-8


def test_coupled_long_beta_matches_oracle():
    """lambda = 0.8 at beta = 20 on a 6x6 lattice: GPU strings against the
    oracle's, G and Re ln_cw."""
    m, o, ft, g = _pair(epsocz_small, L=6, ntime=200, ngroup=10, alpha=0.3)
    g.init_g(1)
    go, lo = ft.init_g(1)
    assert rel_fro(g.g(), go) < 1e-9
    w = g.state()["ln_cw"]
    assert abs(w.real - lo.real) <= W_TOL * abs(lo.real)


def test_scratch_both_directions_without_updates():
    """A backward then a forward pass of wraps with a recompute every ngroup
    slices: the wrapped G and the GPU recompute agree (err_g), and each
    recompute matches the oracle's at the same slice."""
    m, o, ft, g = _pair(epsocz_small, ntime=40, ngroup=10, alpha=0.3, bc=(1.0, 1.0))
    g.init_g(1)
    _, lo = ft.init_g(1)
    npf = len(m.pf)
    for tc in range(1, m.ntime + 1):
        t = m.ntime - tc + 1
        for pf in range(npf, 0, -1):
            g.right_evolve_g(t, pf)
        if tc % m.ngroup == 0:
            e = g.get_g_scratch(t, False)
            ft.get_g_scratch(t, False)
            assert e[0] < 1e-10 and e[1] <= 1e-9 * abs(lo.real)
            assert rel_fro(g.g(), ft.g_h) < G_TOL, (t, rel_fro(g.g(), ft.g_h))
    for tc in range(1, m.ntime + 1):
        for pf in range(1, npf + 1):
            g.left_evolve_g(tc, pf)
        if tc % m.ngroup == 0:
            e = g.get_g_scratch_ft(tc + 1, True)
            ft.get_g_scratch(tc + 1, True)
            assert e[0] < 1e-10 and e[1] <= 1e-9 * abs(lo.real)
            assert rel_fro(g.g(), ft.g_h) < G_TOL, (tc, rel_fro(g.g(), ft.g_h))


def _oracle_ft_sweep(m, o, ft, loop):
    """One sweep of src/Main_PQMC.f90:99-154 on the oracle with the
    finite-temperature recompute (no measurement)."""
    forward = loop % 2 == 0
    npf = len(m.pf)
    for tc in range(1, m.ntime + 1):
        if not forward:
            t = m.ntime - tc + 1
            for pf in range(npf, 0, -1):
                o.right_evolve_g(t, pf)
                if m.spec.pfs[pf - 1].v_exist:
                    o.update_phonon_field(pf, t)
        else:
            t = tc
            for pf in range(1, npf + 1):
                if m.spec.pfs[pf - 1].v_exist:
                    o.update_phonon_field(pf, t)
                o.left_evolve_g(t, pf)
        if tc % m.ngroup == 0:
            ft.get_g_scratch(t + 1 if forward else t, forward, o.g(), None)
            o.set_g(ft.g_h)


def test_ft_sweeps_match_oracle():
    """Two sweeps (backward, forward) at finite temperature: the GPU sweep
    driver with the FT recompute against the oracle's update and wraps with
    the CPU FT recompute.  Same ran2 stream, so the accept/reject sequence,
    the field and the counters agree exactly; G within 1e-10 after each
    sweep; the fast-update error stays small."""
    m, o, ft, g = _pair(epsocz_small, ntime=40, ngroup=10)
    g.init_g(1)
    go, _ = ft.init_g(1)
    o.set_g(go)
    for loop in (1, 2):
        g.sweep(loop, 1)
        _oracle_ft_sweep(m, o, ft, loop)
        so, sg = o.state(), g.state()
        assert sg["rng"] == so["rng"], loop
        assert (sg["positive_accept"], sg["negative_accept"]) == (so["positive_accept"], so["negative_accept"])
        assert np.array_equal(g.field(), o.field())
        assert rel_fro(g.g(), o.g()) < G_TOL, loop
    assert so["positive_accept"] > 0 and so["negative_accept"] > 0
    assert sg["err_g_rel_max"] < 1e-9


def test_switch_back_to_projector():
    """proj = 1 again: init_g is init_g_T0 and G matches a fresh chain's."""
    from pqmc_allinone_gb300.engine import PqmcChain
    m, o, ft, g = _pair(epsocz_small, ntime=20, ngroup=5)
    g.init_g(1)
    g.set_temperature(True)
    assert g.proj()
    g.init_g(1)
    ref = PqmcChain(m, field=g.field(), rng_words=SEED_WORDS)
    ref.init_expkv()
    ref.init_g(1)
    assert rel_fro(g.g(), ref.g()) < 1e-14


def test_batch_chains_stay_projector():
    from pqmc_allinone_gb300.engine import PqmcBatch
    from pqmc_allinone_gb300.rng import seed_words
    m, f = epsocz_small(ntime=20, ngroup=5)
    b = PqmcBatch([m] * 2, [f] * 2, [seed_words(1), seed_words(2)], precision=1)
    with pytest.raises(RuntimeError, match="projector"):
        b.chains[0].set_temperature(False)
    b.close()
