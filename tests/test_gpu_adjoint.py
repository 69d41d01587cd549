"""Differentiable projector log-weight: pqmc_logweight_grad and the
torch.autograd.Function over it, against central finite differences of
cal_new_weight_T0 (src/mod_evolution.f90:359-408) at h = 1e-6.

Tolerance: W = Re ln_cw is O(10..100); a central difference at h = 1e-6 has
roundoff ~ eps |W| / h ~ 1e-8 and truncation ~ h^2 W''' ~ 1e-12, so the
comparison uses |g - fd| <= 1e-6 + 1e-6 |fd|.
"""
import numpy as np
import pytest

from tests.helpers import SEED_WORDS, epsoc_model, epsocz_small, general_bond_model, rel_fro

pytestmark = pytest.mark.gpu

H = 1e-6
ATOL = 1e-6
RTOL = 1e-6

MODELS = [
    ("epsocz", epsocz_small, {}),
    ("epsocz_soc", epsocz_small, {"alpha": 0.3, "bc": (1.0, 1.0)}),
    ("epsoc", epsoc_model, {}),
    ("general", general_bond_model, {}),
]


def _chain(m, f):
    from pqmc_allinone_gb300.engine import PqmcChain
    ch = PqmcChain(m, field=f, rng_words=SEED_WORDS)
    ch.init_expkv()
    ch.init_g(1)
    return ch


def _grad(ch, m):
    import torch
    buf = torch.empty((m.ntime, m.n_bf), dtype=torch.float64, device="cuda")   # (n_bf, ntime) column-major
    w = ch.logweight_grad_device(buf.data_ptr())
    torch.cuda.synchronize()
    return w, buf.cpu().numpy().T.copy()


def _weight(ch, f):
    ch.set_field(f)
    ch.init_expkv()
    ch.init_g(1)
    return ch.cal_new_weight().real


@pytest.mark.parametrize("name,builder,kw", MODELS, ids=[m[0] for m in MODELS])
def test_grad_vs_fd(name, builder, kw):
    m, f = builder(ntime=20, ngroup=5, **kw)
    ch = _chain(m, f)
    w, g = _grad(ch, m)
    assert abs(w.real - _weight(ch, f)) <= 1e-9 * abs(w.real) + 1e-9
    rng = np.random.default_rng(11)
    idx = [(int(rng.integers(m.n_bf)), int(rng.integers(m.ntime))) for _ in range(12)]
    idx += [(0, 0), (m.n_bf - 1, m.ntime - 1), (m.n_bf // 2, m.ngroup - 1), (1, m.ngroup)]
    for (b, t) in idx:
        fp = f.copy(); fp[b, t] += H
        fm = f.copy(); fm[b, t] -= H
        fd = (_weight(ch, fp) - _weight(ch, fm)) / (2 * H)
        assert abs(g[b, t] - fd) <= ATOL + RTOL * abs(fd), (name, b, t, g[b, t], fd)


def test_grad_all_entries_vs_oracle_fd():
    """Every entry of a small field against finite differences of the FP64
    oracle's cal_new_weight (independent of the device code)."""
    from oracle.oracle import OracleChain
    m, f = epsocz_small(ntime=8, ngroup=4, alpha=0.3, bc=(1.0, 1.0))
    ch = _chain(m, f)
    _, g = _grad(ch, m)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS)

    def wo(x):
        o.set_field(x)
        o.init_expkv()
        o.init_g(1)
        return o.cal_new_weight().real

    fd = np.zeros_like(g)
    for b in range(m.n_bf):
        for t in range(m.ntime):
            fp = f.copy(); fp[b, t] += H
            fm = f.copy(); fm[b, t] -= H
            fd[b, t] = (wo(fp) - wo(fm)) / (2 * H)
    assert np.all(np.abs(g - fd) <= ATOL + RTOL * np.abs(fd)), np.max(np.abs(g - fd))
    assert np.abs(g).max() > 1e-3     # the field does move the weight


@pytest.mark.parametrize("name,builder,kw", MODELS, ids=[m[0] for m in MODELS])
def test_grad_vs_fp64_trace_formula(name, builder, kw):
    """Every entry against the FP64 Green's-function trace formula
    c Re Tr[g dE E^-1] evaluated directly on the CPU (oracle/trace_gradient.py:
    the oracle's propagators, unstabilised dense G, no code shared with the
    device adjoint).  Both are exact formulas for the same derivative, so the
    tolerance is far below the finite-difference one: 1e-9 absolute plus
    1e-7 of the largest entry (the entries are O(1e-2))."""
    from oracle.trace_gradient import logweight_grad_trace
    m, f = builder(ntime=20, ngroup=5, **kw)
    ch = _chain(m, f)
    w, g = _grad(ch, m)
    wt, gt, _ = logweight_grad_trace(m, f, SEED_WORDS)
    assert abs(w.real - wt) <= 1e-9 * abs(wt) + 1e-9
    assert np.abs(gt).max() > 1e-3
    assert np.abs(g - gt).max() <= 1e-9 + 1e-7 * np.abs(gt).max(), (name, np.abs(g - gt).max())


def test_grad_leaves_state():
    m, f = epsocz_small(ntime=20, ngroup=5)
    ch = _chain(m, f)
    g0 = ch.g()
    q0 = [ch.qd(b) for b in range(1, m.nblock + 1)]
    _grad(ch, m)
    assert rel_fro(ch.g(), g0) == 0.0
    for b in range(1, m.nblock + 1):
        q, d = ch.qd(b)
        assert np.array_equal(q, q0[b - 1][0]) and np.array_equal(d, q0[b - 1][1])
    # the fast-update path keeps working from the same G
    ch.sweep(1, 1)


def test_autograd_function():
    import torch
    from pqmc_allinone_gb300.autograd import log_weight
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f0 = epsocz_small(ntime=8, ngroup=4)
    _, f1 = epsocz_small(ntime=8, ngroup=4, seed=2)
    chains = [PqmcChain(m, field=f0, rng_words=SEED_WORDS), PqmcChain(m, field=f1, rng_words=SEED_WORDS)]
    x = torch.tensor(np.stack([f0, f1]), dtype=torch.float64, device="cuda", requires_grad=True)
    w = log_weight(x, chains)
    ref = [_weight(_chain(m, fi), fi) for fi in (f0, f1)]
    assert np.allclose(w.detach().cpu().numpy(), ref, rtol=1e-10, atol=1e-10)
    (w * torch.tensor([1.0, -2.0], dtype=torch.float64, device="cuda")).sum().backward()
    _, g0 = _grad(_chain(m, f0), m)
    _, g1 = _grad(_chain(m, f1), m)
    gx = x.grad.cpu().numpy()
    assert np.allclose(gx[0], g0, rtol=1e-12, atol=1e-12)
    assert np.allclose(gx[1], -2.0 * g1, rtol=1e-12, atol=1e-12)


def test_autograd_gradcheck():
    import torch
    from pqmc_allinone_gb300.autograd import LogWeight
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f = epsocz_small(ntime=4, ngroup=2)
    chains = [PqmcChain(m, field=f, rng_words=SEED_WORDS)]
    x = torch.tensor(f[None], dtype=torch.float64, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda y: LogWeight.apply(y, chains), (x,), eps=H, atol=1e-5, rtol=1e-4)


def test_c5_full_size_fd_and_trace_formula():
    """The differentiable configuration at its size: 10x10 spin-orbit lattice
    (Ns = 200, Nup = 100, 200 bonds), Lt = 400, dtau = 0.1, x ~ N(0, 0.5^2)
    from seeds 5000 + i, checkpoints every ngroup = 10 slices.  For two
    chains: central finite differences (h = 1e-6, FP64 weights of the
    device) on 64 random entries each, and every entry against the FP64
    trace formula on the CPU (stabilised form, oracle/trace_gradient.py).
    The gradient is formed in FP64 throughout (no FP32 accumulation).  At
    this size |W| is large, so the difference's roundoff, ~ a few eps |W| / h,
    sets its tolerance: 1e-6 + 1e-6 |fd| + 50 eps |W| / h; the trace formula
    carries no such noise and keeps 1e-9 + 1e-7 of the largest entry."""
    from oracle.trace_gradient import logweight_grad_trace_stable
    from pqmc_allinone_gb300 import model as M
    spec = M.epsocz_spec(10, lam=0.8, alpha=0.3, ntime=400, ngroup=10, filling=0.5, jump_distance=0.5)
    m = M.build_model(spec, twist_seed=11, twist=1e-3)
    assert (m.ns, m.nelec, m.n_bf, m.ntime) == (200, 100, 200, 400)
    for i in range(2):
        f = M.field_gaussian(m, 5000 + i)
        ch = _chain(m, f)
        w, g = _grad(ch, m)
        assert abs(w.real - _weight(ch, f)) <= 1e-9 * abs(w.real)
        gt = logweight_grad_trace_stable(m, f, SEED_WORDS)
        assert np.abs(g - gt).max() <= 1e-9 + 1e-7 * np.abs(gt).max(), np.abs(g - gt).max()
        rng = np.random.default_rng(5000 + i)
        fd_noise = 50.0 * np.finfo(np.float64).eps * abs(w.real) / H
        for _ in range(64):
            b, t = int(rng.integers(m.n_bf)), int(rng.integers(m.ntime))
            fp = f.copy(); fp[b, t] += H
            fm = f.copy(); fm[b, t] -= H
            fd = (_weight(ch, fp) - _weight(ch, fm)) / (2 * H)
            assert abs(g[b, t] - fd) <= ATOL + RTOL * abs(fd) + fd_noise, (b, t, g[b, t], fd, w.real)
        ch.close()
