"""The FP64 trace-formula gradient of the projector log-weight
(oracle/trace_gradient.py), which the GPU adjoint is checked against, pinned
on the CPU: its value equals the oracle's cal_new_weight_T0
(src/mod_evolution.f90:359-408) and every entry of its gradient equals a
central finite difference of that weight, for the three propagator forms
(EPSOCZ closed form with a static spin-orbit term and twisted boundaries,
EPSOC closed form under TR_weight, general expm, and the latter with
ncopy = 2)."""
import numpy as np
import pytest

from tests.helpers import SEED_WORDS, epsoc_model, epsocz_small, general_bond_model

H = 1e-6


def spin_half_bond_model(ntime=8, ngroup=4):
    """The bond model with spin 1/2 as ncopy = 2 (weight det^2)."""
    import dataclasses
    from pqmc_allinone_gb300 import model as M
    m, f = general_bond_model(ntime=ntime, ngroup=ngroup)
    m2 = M.build_model(dataclasses.replace(m.spec, ncopy=2), twist_seed=3, twist=1e-3)
    return m2, f


CASES = [
    ("epsocz_soc", epsocz_small, {"alpha": 0.3, "bc": (1.0, 1.0)}),
    ("epsoc", epsoc_model, {}),
    ("general", general_bond_model, {}),
    ("general_ncopy2", spin_half_bond_model, {}),
]


@pytest.mark.parametrize("name,builder,kw", CASES, ids=[c[0] for c in CASES])
def test_trace_formula_vs_oracle_fd(name, builder, kw):
    from oracle.oracle import OracleChain
    from oracle.trace_gradient import logweight_grad_trace
    m, f = builder(ntime=8, ngroup=4, **kw)
    w, g, dets = logweight_grad_trace(m, f, SEED_WORDS)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)

    def wo(x):
        o.set_field(x)
        o.init_expkv()
        o.init_g(1)
        return o.cal_new_weight().real

    assert abs(w - wo(f)) <= 1e-12 * abs(w) + 1e-12
    # det(P^H B P) is the same at every position of the string
    logs = np.array([d[1] for d in dets])
    assert logs.max() - logs.min() < 1e-10
    fd = np.zeros_like(g)
    for b in range(m.n_bf):
        for t in range(m.ntime):
            fp = f.copy(); fp[b, t] += H
            fm = f.copy(); fm[b, t] -= H
            fd[b, t] = (wo(fp) - wo(fm)) / (2 * H)
    # central differences at h = 1e-6 of W = O(10): roundoff ~ 1e-9
    assert np.abs(g - fd).max() <= 1e-7, (name, np.abs(g - fd).max())
    assert np.abs(g).max() > 1e-3


def test_stabilised_trace_formula_matches_dense():
    """The stabilised trace formula (re-orthonormalised factors, right
    factors checkpointed per block and rebuilt) gives the dense one's
    gradient on a short string where the dense form is well conditioned."""
    from oracle.trace_gradient import logweight_grad_trace, logweight_grad_trace_stable
    m, f = epsocz_small(ntime=20, ngroup=5, alpha=0.3, bc=(1.0, 1.0))
    _, gd, _ = logweight_grad_trace(m, f, SEED_WORDS)
    gs = logweight_grad_trace_stable(m, f, SEED_WORDS)
    assert np.abs(gs - gd).max() <= 1e-10 + 1e-9 * np.abs(gd).max()
