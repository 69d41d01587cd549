"""Checkpoint/resume: a chain (or batch) saved after an even sweep and
restored into a fresh handle continues with the same accept/reject sequence
as the original run (fields bit-identical), because the restore rebuilds
expKV and G from the exact field (init_expKV, init_g_T0(1)) and takes the
saved ran2 state and counters."""
import numpy as np
import pytest

from pqmc_allinone_gb300 import checkpoint as ck
from pqmc_allinone_gb300.rng import seed_words
from tests.helpers import epsocz_small, rel_fro

pytestmark = pytest.mark.gpu


def test_chain_resume(tmp_path):
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=31)
    a = PqmcChain(m, field=f, rng_words=seed_words(310))
    a.init_expkv()
    a.init_g(1)
    a.sweep(1, 2)
    p = str(tmp_path / "chain.npz")
    ck.save_checkpoint(p, [a], 2)
    a.sweep(3, 2)
    b = PqmcChain(m, field=np.zeros_like(f), rng_words=seed_words(999))
    nxt = ck.restore_chain(b, ck.load_checkpoint(p))
    assert nxt == 3
    b.sweep(nxt, 2)
    assert np.array_equal(a.field(), b.field())
    sa, sb = a.state(), b.state()
    assert sa["positive_accept"] == sb["positive_accept"] and sa["negative_accept"] == sb["negative_accept"]
    assert sa["rng"] == sb["rng"]
    assert rel_fro(b.g(), a.g()) < 1e-12


def test_uneven_batch_resume(tmp_path):
    from pqmc_allinone_gb300.engine import PqmcBatch
    ms = []
    for i, (L, nt) in enumerate([(4, 20), (6, 40), (4, 20)]):
        m, f = epsocz_small(L=L, ntime=nt, ngroup=10, lam=0.8, alpha=0.3, seed=40 + i)
        ms.append((m, f, seed_words(400 + i)))
    mk = lambda: PqmcBatch([m for m, _, _ in ms], [f for _, f, _ in ms], [w for _, _, w in ms], precision=1)
    a = mk()
    a.set_graphs(True)
    a.init()
    for loop in (1, 2):
        a.sweep(loop)
    p = str(tmp_path / "batch.npz")
    ck.save_checkpoint(p, a.chains, 2)
    for loop in (3, 4):
        a.sweep(loop)
    b = mk()
    b.set_graphs(True)
    nxt = ck.restore_batch(b, ck.load_checkpoint(p))
    for loop in (nxt, nxt + 1):
        b.sweep(loop)
    for ca, cb in zip(a.chains, b.chains):
        assert np.array_equal(ca.field(), cb.field())
        assert ca.state()["positive_accept"] == cb.state()["positive_accept"]
        assert rel_fro(cb.g(), ca.g()) < 1e-12
    a.close()
    b.close()


def test_chain_resume_matches_uninterrupted_oracle(tmp_path):
    """A GPU chain checkpointed after sweep 2, restored into a fresh handle
    and run for sweeps 3-4 against the FP64 oracle run for sweeps 1-4 with
    no interruption (src/Main_PQMC.f90:355-369 reads the field back; the
    saved ran2 state and counters continue the stream): the same
    accept/reject sequence (field, counters, ran2 state) and G within 1e-10."""
    from oracle.oracle import OracleChain
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.8, alpha=0.3, seed=33)
    w = seed_words(330)
    a = PqmcChain(m, field=f, rng_words=w)
    a.init_expkv()
    a.init_g(1)
    a.sweep(1, 2)
    p = str(tmp_path / "chain.npz")
    ck.save_checkpoint(p, [a], 2)
    a.close()
    b = PqmcChain(m, field=np.zeros_like(f), rng_words=seed_words(999))
    nxt = ck.restore_chain(b, ck.load_checkpoint(p))
    b.sweep(nxt, 2)
    o = OracleChain(m, field=f, seed_words=w, meas=False)
    o.init_expkv()
    o.init_g(1)
    o.sweep(1, 4)
    so, sb = o.state(), b.state()
    assert np.array_equal(b.field(), o.field())
    assert (sb["positive_accept"], sb["negative_accept"]) == (so["positive_accept"], so["negative_accept"])
    assert sb["rng"] == so["rng"]
    assert rel_fro(b.g(), o.g()) < 1e-10
