"""Global moves on the device against the oracle: update_global (new
field, cal_new_weight_T0 of it, Metropolis test, restore on rejection) and
the driver's global step inside pqmc_sweep (Main_PQMC.f90:87-96), from the
same field and ran2 state."""
import numpy as np
import pytest

from oracle import global_update as og
from pqmc_allinone_gb300.abi import global_params
from pqmc_allinone_gb300.rng import seed_words
from tests.helpers import epsocz_small, rel_fro

pytestmark = pytest.mark.gpu


def _pair(m, f, w):
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcChain
    ch = PqmcChain(m, field=f, rng_words=w)
    ch.init_expkv()
    ch.init_g(1)
    oc = OracleChain(m, field=f, seed_words=w, meas=False)
    oc.init_expkv()
    oc.init_g(1)
    return ch, oc


@pytest.mark.parametrize("kind,kw,dist", [
    (og.KSPACE, {}, 0.05), (og.KSPACE, {}, 40.0), (og.ROTATE, {}, 1.0), (og.KSPACE_TIME, {}, 0.05),
    (og.KSPACE_TIME, {}, 40.0), (og.EXCHANGE, {"n_global_update": 2}, 1.0),
    (og.SINGLE, {"shift": True}, 0.5), (og.SINGLE, {"flip": True}, 1.0)])
def test_update_global_matches_oracle(kind, kw, dist):
    m, f = epsocz_small(L=4, ntime=200 if kind == og.KSPACE_TIME else 40, ngroup=10, lam=0.8, alpha=0.3,
                        seed=17)
    gp = global_params(m, global_update_distance=dist, **kw)
    outcomes = []
    for k in range(4):
        w = seed_words(500 + k)
        ch, oc = _pair(m, f, w)
        ch.set_global(gp)
        ln0 = ch.state()["ln_cw"]
        acc = ch.update_global(kind)
        rng = og.Ran2(w)
        acc_o, ln_o = og.update_global(oc, m, gp, kind, oc.state()["ln_cw"], rng)
        assert acc == acc_o
        assert ch.state()["rng"] == rng.words
        assert np.allclose(ch.field(), oc.field(), rtol=0, atol=1e-13)
        ln1 = ch.state()["ln_cw"]
        if acc:
            assert abs(ln1.real - ln_o.real) <= 1e-8 * abs(ln_o.real)
        else:
            assert ln1 == ln0 and np.array_equal(ch.field(), f)
        assert ch.global_counters() == (int(acc), int(not acc))
        outcomes.append(acc)
        ch.close()
    if dist >= 40.0:
        assert not all(outcomes)


def test_global_step_in_sweep_matches_oracle():
    """pqmc_sweep with global moves enabled: before every backward sweep
    (global_update_loop=2) the kspace, rotate and kspace_time moves and
    init_g_T0(1) after an acceptance; fields and accept counts follow the
    oracle driven the same way."""
    m, f = epsocz_small(L=4, ntime=200, ngroup=10, lam=0.8, alpha=0.3, seed=23)
    gp = global_params(m, global_update_distance=0.05)
    w = seed_words(321)
    ch, oc = _pair(m, f, w)
    ch.set_global(gp)
    n_acc = 0
    for loop in (1, 2, 3, 4):
        ch.sweep(loop, 1)
        n, words = og.global_step(oc, m, gp, loop, oc.state()["ln_cw"], oc.state()["rng"])
        n_acc += n
        oc.sweep(loop, 1)
        assert np.allclose(ch.field(), oc.field(), rtol=0, atol=1e-12), loop
        assert ch.state()["positive_accept"] == oc.state()["positive_accept"]
    assert ch.global_counters()[0] == n_acc
    assert sum(ch.global_counters()) == 6          # 3 moves before sweeps 1 and 3
    assert rel_fro(ch.g(), oc.g()) < 1e-9


def test_batch_sweep_runs_global_steps():
    """A mixed batch whose chain 0 has global moves enabled: the batched
    sweep takes the driver's global step for that chain only, and the chain
    stays consistent (G after the sweeps matches the FP64 oracle on its
    field)."""
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i in range(2):
        m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=60 + i)
        ms.append((m, f, seed_words(600 + i)))
    b = PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    b.init()
    b.chains[0].set_global(global_params(ms[0][0], global_update_distance=0.05))
    for loop in (1, 2, 3, 4):
        b.sweep(loop)
    assert sum(b.chains[0].global_counters()) == 6 and b.chains[1].global_counters() == (0, 0)
    for (m, _, w), ch in zip(ms, b.chains):
        o = OracleChain(m, field=ch.field(), seed_words=w, meas=False)
        o.init_expkv()
        o.init_g(1)
        assert rel_fro(ch.g(), o.g()) < 1e-10
    b.close()
