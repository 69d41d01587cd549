"""The finite-temperature oracle (oracle/finite_t.py) against known answers.

init_g_FT / cal_g_and_det_FT / get_g_scratch_FT / cal_new_weight_FT of
src/mod_evolution.f90:409-785, restated with the corrections the module
header lists, must give
  * g_h = 1 - (1 + B(beta,0))^-1 and ln_cw = log det(1 + B(beta,0)) from one
    dense product at short beta;
  * the free-fermion answer (lambda = 0: every slice propagator the same
    matrix, diagonalised once) at long beta, where the dense product is
    useless;
  * scratch recomputes that agree with G wrapped slice by slice through a
    whole backward and forward pass (the err_fast invariant, :720-744);
and the reference's own final call of init_g_FT (rmat^H and block nblock-1
on both sides, :485-489) does not.
"""
import numpy as np
import pytest

from tests.helpers import SEED_WORDS, epsocz_small, general_bond_model, rel_fro


def _oracle(m, f):
    from oracle.oracle import OracleChain
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)
    o.init_expkv()
    return o


@pytest.mark.parametrize("builder,kw", [
    (epsocz_small, {"ntime": 20, "ngroup": 5}),
    (epsocz_small, {"ntime": 20, "ngroup": 5, "alpha": 0.3, "bc": (1.0, 1.0)}),
    (general_bond_model, {"ntime": 20, "ngroup": 4}),
], ids=["epsocz", "epsocz_soc", "general"])
def test_init_g_matches_dense(builder, kw):
    from oracle.finite_t import FiniteT, dense_g_and_weight
    m, f = builder(**kw)
    o = _oracle(m, f)
    ft = FiniteT(o)
    g, ln = ft.init_g(1)
    gd, lnd = dense_g_and_weight(o)
    assert rel_fro(g, gd) < 1e-11
    assert abs(ln.real - lnd.real) <= 1e-10 * abs(lnd.real) + 1e-10
    assert abs(np.exp(1j * ln.imag) - np.exp(1j * lnd.imag)) < 1e-9
    assert abs(ft.cal_new_weight().real - ln.real) <= 1e-10 * abs(ln.real) + 1e-10


def test_reference_final_call_is_not_the_known_answer():
    """init_g_FT's own final call (lmat = rmat^H, block nblock-1 as both the
    left and the right factors) computes (1 + B B^H)^-1, not (1 + B)^-1."""
    from oracle.finite_t import FiniteT, cal_g_and_det_ft, dense_g_and_weight
    m, f = epsocz_small(ntime=20, ngroup=5)
    o = _oracle(m, f)
    ft = FiniteT(o)
    ft.init_g(1)
    nb = ft.nblock
    rmat = ft.q[nb - 1]
    g_ref, _ = cal_g_and_det_ft(m, rmat.conj().T, rmat, ft.d[nb - 1], ft.d[nb - 1],
                                ft.r[nb - 1].conj().T, ft.r[nb - 1])
    gd, _ = dense_g_and_weight(o)
    assert rel_fro(g_ref, gd) > 1e-3


@pytest.mark.parametrize("ntime,ngroup", [(200, 10), (400, 20), (1000, 10)])
def test_free_fermions_long_beta(ntime, ngroup):
    """lambda = 0: B(beta,0) = B(1)^ntime, g_h from the eigenvectors of B(1);
    beta = 20, 40 and 100 (the dense product has a condition number beyond
    1e30)."""
    from oracle.finite_t import FiniteT, free_fermion_g
    m, f = epsocz_small(L=4, ntime=ntime, ngroup=ngroup, lam=0.0, alpha=0.3)
    o = _oracle(m, f)
    ft = FiniteT(o)
    g, ln = ft.init_g(1)
    gf, ref = free_fermion_g(o)
    assert rel_fro(g, gf) < 1e-9
    assert abs(ln.real - ref) <= 1e-10 * abs(ref) + 1e-9


def test_scratch_matches_wrapped_g_both_directions():
    """After init_g (G at beta) a backward pass wraps G down slice by slice
    (right_evolve two-way, families n_pf..1) and recomputes it every ngroup
    slices from the left string; a forward pass then wraps it up again and
    recomputes from the right string.  No updates: the wrapped and the
    recomputed G agree to rounding, and so do the weights."""
    from oracle.finite_t import FiniteT
    m, f = epsocz_small(ntime=40, ngroup=10, alpha=0.3, bc=(1.0, 1.0))
    o = _oracle(m, f)
    ft = FiniteT(o)
    g, ln = ft.init_g(1)
    o.set_g(g)
    npf = len(m.pf)
    worst = 0.0
    for tc in range(1, m.ntime + 1):          # backward (Main_PQMC.f90:101-116)
        t = m.ntime - tc + 1
        for pf in range(npf, 0, -1):
            o.right_evolve_g(t, pf)
        if tc % m.ngroup == 0:
            eg, ew = ft.get_g_scratch(t, False, o.g(), ln)
            worst = max(worst, rel_fro(o.g(), ft.g_h))
            assert ew <= 1e-9 * abs(ln.real) + 1e-9
            o.set_g(ft.g_h)
    for tc in range(1, m.ntime + 1):          # forward (:119-129)
        t = tc
        for pf in range(1, npf + 1):
            o.left_evolve_g(t, pf)
        if tc % m.ngroup == 0:
            eg, ew = ft.get_g_scratch(t + 1, True, o.g(), ln)
            worst = max(worst, rel_fro(o.g(), ft.g_h))
            assert ew <= 1e-9 * abs(ln.real) + 1e-9
            o.set_g(ft.g_h)
    assert worst < 1e-10, worst


def test_svd_strings_lose_the_small_scales(monkeypatch):
    """The reference decomposes the strings with the SVD (udv, :470): on the
    same free-fermion chain at beta = 20 that loses the small scales of the
    column-graded products, so G and Re ln det come out wrong; the pivoted
    QR the oracle uses instead is exact to rounding (test above)."""
    import oracle.finite_t as F
    m, f = epsocz_small(L=4, ntime=200, ngroup=10, lam=0.0, alpha=0.3)
    o = _oracle(m, f)
    monkeypatch.setattr(F, "udv_strings", lambda a: (lambda u, s, vh: (u, s, vh))(*F.udv(a)))
    ft = F.FiniteT(o)
    g, ln = ft.init_g(1)
    gf, ref = F.free_fermion_g(o)
    assert rel_fro(g, gf) > 0.1 and abs(ln.real - ref) > 1.0
