"""Global moves (update_global / generate_newfield_global,
src/mod_update.f90:250-467): the library's host-side field generation
(pqmc_global_generate, no GPU needed) against the oracle's restatement, draw
by draw, for every update_type; and the invariants of each move."""
import numpy as np
import pytest

from oracle import global_update as og
from pqmc_allinone_gb300.abi import global_params
from pqmc_allinone_gb300.engine import global_generate
from pqmc_allinone_gb300.rng import seed_words
from tests.helpers import epsocz_small

CASES = [
    ("kspace", og.KSPACE, {}),
    ("kspace_time", og.KSPACE_TIME, {}),
    ("rotate", og.ROTATE, {}),
    ("exchange", og.EXCHANGE, {"n_global_update": 3}),
    ("flip", og.SINGLE, {"flip": True, "n_global_update": 2}),
    ("shift", og.SINGLE, {"shift": True, "n_global_update": 2}),
]


def _model(ntime=40):
    return epsocz_small(L=4, ntime=ntime, ngroup=10, lam=0.8, alpha=0.3, seed=5)


@pytest.mark.parametrize("name,kind,kw", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_generate_matches_oracle(name, kind, kw, seed):
    m, f = _model(ntime=400 if kind == og.KSPACE_TIME else 40)
    gp = global_params(m, global_update_distance=1.0, **kw)
    w = seed_words(70 + seed)
    f1, ph1, a1, b1, w1 = global_generate(m, gp, kind, w, f)
    rng = og.Ran2(w)
    f2, ph2, a2, b2 = og.generate(m, gp, kind, rng, f)
    assert w1 == rng.words and (a1, b1) == (a2, b2)
    assert np.allclose(f1, f2, rtol=0, atol=1e-14), np.abs(f1 - f2).max()
    assert abs(ph1 - ph2) <= 1e-11 * (1 + abs(ph2))
    assert not np.array_equal(f1, f)


def test_move_invariants():
    m, f = _model(ntime=400)
    gp = global_params(m)
    w = seed_words(5)
    # rotate keeps x^2 + y^2 of every cell and slice and has no action term
    fr, ph, _, _, _ = global_generate(m, gp, og.ROTATE, w, f)
    r0 = f[0::2] ** 2 + f[1::2] ** 2
    r1 = fr[0::2] ** 2 + fr[1::2] ** 2
    assert np.allclose(r0, r1, rtol=1e-13) and ph == 0.0
    # kspace adds one staggered pattern to every slice; omega=1 action change
    # 0.5*D*sum(x'^2-x^2)*(-delt) (no kinetic change)
    fk, ph, t0, t1, _ = global_generate(m, gp, og.KSPACE, w, f)
    d = fk - f
    assert (t0, t1) == (1, m.ntime) and np.allclose(d, d[:, :1], atol=1e-14)
    # +-amplitude*cos(pi_sp*(x+y)) on every bond: equal up to cos(n*pi_sp) ~ 1 - O(1e-14)
    assert abs(np.abs(d[:, 0]).max() - np.abs(d[:, 0]).min()) < 1e-12
    assert np.isclose(ph, -m.spec.delt * 0.5 * m.D * np.sum(fk ** 2 - f ** 2), rtol=1e-10)
    # kspace_time: slices start..ntime (start in 1..ntime/2), untouched before
    ft, ph, t0, t1, _ = global_generate(m, gp, og.KSPACE_TIME, w, f)
    assert 1 <= t0 <= m.ntime // 2 and t1 == m.ntime
    assert np.array_equal(ft[:, :t0 - 1], f[:, :t0 - 1])
    # exchange is a permutation of time lines
    fe, ph, _, _, _ = global_generate(m, gp | {"n_global_update": 4}, og.EXCHANGE, w, f)
    assert ph == 0.0 and np.array_equal(np.sort(fe, axis=0), np.sort(f, axis=0))
    # flip negates one time line and costs only the bias term (zero here)
    ff, ph, _, _, _ = global_generate(m, gp | {"flip": 1}, og.SINGLE, w, f)
    rows = np.where(np.any(ff != f, axis=1))[0]
    assert len(rows) == 1 and np.array_equal(ff[rows[0]], -f[rows[0]]) and ph == 0.0


def test_generate_errors():
    from pqmc_allinone_gb300.abi import PqmcError
    m, f = _model()
    gp = global_params(m)
    with pytest.raises(PqmcError):
        global_generate(m, gp, og.SINGLE, seed_words(1), f)          # neither flip nor shift
    with pytest.raises(PqmcError):
        global_generate(m, gp, 9, seed_words(1), f)
    with pytest.raises(PqmcError):
        global_generate(m, gp | {"n_cell": gp["n_cell"] - 1}, og.KSPACE, seed_words(1), f)
