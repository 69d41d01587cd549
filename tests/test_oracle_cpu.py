"""CPU tests of the oracle and the host-side set-up (no GPU)."""
import os

import numpy as np
import pytest

from oracle.oracle import OracleChain, lib, rng_draw
from pqmc_allinone_gb300 import model as M
from pqmc_allinone_gb300.rng import Ran2, seed_words
from tests.helpers import SEED_WORDS, epsoc_model, epsocz_small, general_bond_model, rel_fro

GOLD = os.path.join(os.path.dirname(__file__), "golden")


# ---- ran2 (src/mod_ranstate.f90) --------------------------------------
@pytest.mark.parametrize("seed", [42, 122])
def test_ran2_golden(seed):
    gold = np.load(os.path.join(GOLD, f"ran2_seed{seed}.npy"))
    draws, _ = rng_draw(seed_words(seed), gold.size)
    assert np.array_equal(draws, gold)
    r = Ran2.from_seed(seed)
    py = np.array([r.next() for _ in range(gold.size)], dtype=np.float32)
    assert np.array_equal(py, gold)
    assert gold.min() > 0.0 and gold.max() < 1.0


def test_ran2_seed_words():
    assert seed_words(42) == [42] * 5
    assert seed_words(0)[3:] == [1, 1]
    assert seed_words(-5)[:3] == [4, 4, 4]


# ---- model set-up -------------------------------------------------------
def test_namelist_matches_builder(reference_root):
    nml = os.path.join(reference_root, "input", "model", "EPSOCZ.nml")
    spec = M.spec_from_namelist(open(nml).read())
    m1 = M.build_model(spec, with_slater=False)
    s2 = M.epsocz_spec(tuple(spec.lat_size), lam=spec.ep_parameter, ntime=m1.ntime, ngroup=spec.ngroup,
                       filling=spec.filling, jump_distance=spec.jump_distance, bc_phase=tuple(spec.bc_phase))
    m2 = M.build_model(s2, with_slater=False)
    for a, b in zip(m1.pf, m2.pf):
        assert np.array_equal(a.site_list, b.site_list)
        assert np.array_equal(a.bf_list, b.bf_list)
        assert np.array_equal(a.crossing, b.crossing)
        assert np.allclose(a.bc_phases, b.bc_phases)
    assert np.allclose(m1.kmat, m2.kmat) and np.allclose(m1.vmat, m2.vmat)
    assert m1.ns == 128 and [t.n_pla for t in m1.pf] == [32] * 4


def test_families_partition_sites():
    m, _ = epsocz_small(L=6)
    for t in m.pf:
        s = np.sort(t.site_list.ravel())
        assert np.array_equal(s, np.arange(m.ns))
    bf = np.sort(np.concatenate([t.bf_list for t in m.pf]))
    assert np.array_equal(bf, np.arange(m.n_bf))


def test_k_phase_unitary_and_rel_index():
    m, _ = epsocz_small(L=4)
    kp = m.lat.k_phase
    assert np.allclose(kp @ kp.conj().T, m.lat.n_cell * np.eye(m.lat.n_cell))
    t = M.meas_tables(m)
    rel = t["rel_index"]
    for c1 in range(m.lat.n_cell):
        assert sorted(rel[:, c1]) == list(range(m.lat.n_cell))


def test_slater_orthonormal():
    m, _ = epsocz_small(L=4)
    q = m.slater_q
    assert np.allclose(q.conj().T @ q, np.eye(m.nelec), atol=1e-12)


# ---- dense kernels vs LAPACK conventions (numpy) -------------------------
def test_qdr_matches_lapack():
    import ctypes
    rng = np.random.default_rng(0)
    a = rng.normal(size=(30, 12)) + 1j * rng.normal(size=(30, 12))
    q = np.asfortranarray(a.copy())
    d = np.zeros(12, dtype=np.complex128)
    lib().oracle_qdr(30, 12, q.ctypes.data_as(ctypes.c_void_p), d.ctypes.data_as(ctypes.c_void_p))
    qn, rn = np.linalg.qr(a)
    assert np.allclose(q, qn, atol=1e-12)
    assert np.allclose(d, np.diag(rn), atol=1e-12)
    assert np.allclose(d.imag, 0.0)


def test_ldq_is_adjoint_qr():
    import ctypes
    rng = np.random.default_rng(1)
    a = rng.normal(size=(8, 20)) + 1j * rng.normal(size=(8, 20))
    q = np.asfortranarray(a.copy())
    d = np.zeros(8, dtype=np.complex128)
    lib().oracle_ldq(8, 20, q.ctypes.data_as(ctypes.c_void_p), d.ctypes.data_as(ctypes.c_void_p))
    qn, rn = np.linalg.qr(a.conj().T)
    assert np.allclose(q, qn.conj().T, atol=1e-12)
    assert np.allclose(d, np.diag(rn).conj(), atol=1e-12)


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_det_small_and_inverse(n):
    import ctypes
    rng = np.random.default_rng(n)
    a = np.asfortranarray(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    out = np.zeros(2)
    lib().oracle_det_small(n, a.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
    assert np.isclose(complex(*out), np.linalg.det(a), rtol=1e-13)
    b = a.copy(order="F")
    assert lib().oracle_inverse(n, b.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.allclose(b, np.linalg.inv(a), rtol=1e-12, atol=1e-13)


# ---- expKV: closed forms vs expm (src/mod_phonon_field.f90:451-469) ------
@pytest.mark.parametrize("builder,kind,kw", [
    (epsocz_small, M.EXPKV_EPSOCZ, {}),
    (epsocz_small, M.EXPKV_EPSOCZ_BLOCK, {"alpha": 0.3, "bc": (1.0, 1.0)}),
    (epsoc_model, M.EXPKV_EPSOC, {}),
])
def test_closed_form_matches_expm(builder, kind, kw):
    m, f = builder(**kw)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)
    rng = np.random.default_rng(2)
    for pf in range(len(m.pf)):
        for pla in range(0, m.pf[pf].n_pla, 3):
            for x in rng.normal(0.0, 1.0, size=3):
                for inv in (0, 1):
                    a = o.expkv_single(kind, pf, pla, x, inv)
                    b = o.expkv_single(M.EXPKV_GENERAL, pf, pla, x, inv)
                    assert np.allclose(a, b, atol=1e-13), (pf, pla, x, inv)
                e = o.expkv_single(kind, pf, pla, x, 0) @ o.expkv_single(kind, pf, pla, x, 1)
                assert np.allclose(e, np.eye(m.pf[pf].dim), atol=1e-13)


def test_expm_against_scipy():
    import ctypes
    import scipy.linalg as sl
    rng = np.random.default_rng(3)
    for n in (2, 3, 4):
        h = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        h = 0.3 * (h + h.conj().T)
        for mat in (h, 1j * h):
            a = np.asfortranarray(mat.copy())
            lib().oracle_expm(n, a.ctypes.data_as(ctypes.c_void_p))
            assert np.allclose(a, sl.expm(mat), atol=1e-13)


# ---- invariants of the sweep -----------------------------------------------
@pytest.mark.parametrize("builder,kw", [(epsocz_small, {}), (epsocz_small, {"alpha": 0.3}),
                                        (epsoc_model, {}), (general_bond_model, {})])
def test_fast_vs_scratch(builder, kw):
    """err_fast invariant (src/mod_evolution.f90:179-193): the wrapped and
    updated G and ln_cw agree with the stabilised recompute."""
    m, f = builder(**kw)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)
    o.init_expkv()
    o.init_g(1)
    for loop in range(1, 4):
        o.sweep(loop, 1)
        s = o.state()
        assert s["err_fast_max"] <= 1e-6 + 1e-15
    assert s["positive_accept"] > 0 and s["negative_accept"] > 0
    g = o.g()
    assert np.allclose(g @ g, g, atol=1e-10)          # g_h = R (L R)^-1 L is a projector
    assert abs(np.trace(g) - m.nelec) < 1e-9


def test_projector_known_answer():
    """For a fixed field, G from the stabilised QDR string equals the naive
    R (L R)^-1 L with R = B(ntime..1) P and L = P^H at the left end."""
    m, f = epsocz_small(L=4, ntime=20, ngroup=5, lam=0.8)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)
    o.init_expkv()
    o.init_g(1)
    R = np.asfortranarray(m.slater_q.copy())
    for t in range(1, m.ntime + 1):
        for pf in range(1, len(m.pf) + 1):
            R = o.left_evolve(t, pf, R)
    L = m.slater_q.conj().T
    g_naive = R @ np.linalg.solve(L @ R, L)
    assert rel_fro(o.g(), g_naive) < 1e-10
    ln_naive = np.log(np.linalg.det(L @ R))
    assert abs(o.state()["ln_cw"].real - ln_naive.real) < 1e-9 * abs(ln_naive.real) + 1e-9
    # cal_new_weight_T0 gives the same log-weight
    assert abs(o.cal_new_weight().real - ln_naive.real) < 1e-9 * abs(ln_naive.real) + 1e-9


def test_free_fermions_lambda_zero():
    """lambda = 0: the field drops out of B, G is field independent."""
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.0)
    o1 = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=False)
    o2 = OracleChain(m, field=-3.0 * f, seed_words=SEED_WORDS, meas=False)
    for o in (o1, o2):
        o.init_expkv()
        o.init_g(1)
    assert rel_fro(o1.g(), o2.g()) < 1e-12


def test_golden_sweeps():
    gold = np.load(os.path.join(GOLD, "sweep_epsocz4.npz"))
    m, f = epsocz_small(L=4, ntime=40, ngroup=10, lam=0.8)
    assert np.array_equal(f, gold["field0"])
    o = OracleChain(m, field=f, seed_words=seed_words(42), meas=False)
    o.init_expkv()
    o.init_g(1)
    assert rel_fro(o.g(), gold["g0"]) < 1e-12
    o.sweep(1, 3)
    s = o.state()
    assert np.array_equal(o.field(), gold["field3"])
    assert [s["positive_accept"], s["negative_accept"]] == list(gold["acc3"])
    assert s["rng"] == list(gold["rng3"])
    assert rel_fro(o.g(), gold["g3"]) < 1e-12


def test_measurement_symmetries():
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, bc=(1.0, 1.0))
    o = OracleChain(m, field=f, seed_words=SEED_WORDS)
    o.init_expkv()
    o.init_g(1)
    recs = o.sweep(1, 1, warmup=0, meas_number=0, cap=2)
    assert recs.shape[0] == 1
    nc = m.lat.n_cell
    r = recs[0]
    fields = r[3:3 + 25 * nc].reshape(25, nc)
    kfields = r[3 + 25 * nc:].reshape(25, nc)
    # k-space is the k_phase transform of the r-space record / N_cell
    assert np.allclose(kfields, fields @ m.lat.k_phase.T / nc, atol=1e-12)
    # BF_X equals the field average on the measured slice
    assert np.isclose(r[2].real, o.field()[:, m.ntime // 2 - 1].sum() / nc)


@pytest.mark.parametrize("L", [4, 6])
def test_k_space_matches_fft2(L):
    """The _k observables against numpy's 2-D FFT of their real-space fields,
    the cross-check of pprocess/check_core_data.py:47-111: with the first
    Brillouin zone centred at Gamma (src/mod_lattice.f90:164-202) the k
    index m holds k = 2 pi (m - floor(L/2)) / L, so the record is the
    fftshift of the inverse FFT over the cells."""
    m, f = epsocz_small(L=L, ntime=20, ngroup=10)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS)
    o.init_expkv()
    o.init_g(1)
    r = o.sweep(1, 1, warmup=0, meas_number=0, cap=2)[0]
    nc = m.lat.n_cell
    fields = r[3:3 + 25 * nc].reshape(25, nc)
    kfields = r[3 + 25 * nc:].reshape(25, nc)
    dp = m.lat.cell_dpos
    assert np.abs(fields).max() > 1e-3
    for j in range(25):
        grid = np.zeros((L, L), dtype=np.complex128)
        grid[dp[:, 0], dp[:, 1]] = fields[j]
        want = np.fft.fftshift(np.fft.ifft2(grid))[dp[:, 0], dp[:, 1]]
        assert np.allclose(kfields[j], want, atol=1e-12), j


def test_spin_half_gaussian_bond_model():
    """The 4x4 bond-modulated hopping t(1 - lambda x_b) configuration with
    spin 1/2 as ncopy = 2 (weight det^ncopy, src/mod_update.f90:104) and the
    Gaussian proposal (sigma = 0.3, Box-Muller on two ran2 draws, then the
    Metropolis draw :117): the weight doubles the ncopy = 1 one, a family
    step consumes three draws per plaquette, and the err_fast invariant
    (src/mod_evolution.f90:179-193) holds over Lt = 80."""
    import dataclasses
    from oracle.oracle import rng_draw
    from pqmc_allinone_gb300 import model as M
    m1, f = general_bond_model(L=4, ntime=80, ngroup=10, lam=0.8)
    spec2 = dataclasses.replace(m1.spec, ncopy=2, proposal_kind=M.PROPOSAL_GAUSSIAN, jump_distance=0.3)
    m2 = M.build_model(spec2, twist_seed=3, twist=1e-3)
    assert m2.jump_distance == pytest.approx(0.3)
    o1 = OracleChain(m1, field=f, seed_words=SEED_WORDS, meas=False)
    o2 = OracleChain(m2, field=f, seed_words=SEED_WORDS, meas=False)
    for o in (o1, o2):
        o.init_expkv()
        o.init_g(1)
    assert abs(o2.state()["ln_cw"].real - 2.0 * o1.state()["ln_cw"].real) < 1e-9 * abs(o1.state()["ln_cw"].real)
    # one family step at the first slice: 3 draws per plaquette
    o2.update_phonon_field(1, 1)
    _, words = rng_draw(SEED_WORDS, 3 * m2.pf[0].n_pla)
    assert o2.state()["rng"] == words
    o2.set_rng(SEED_WORDS)
    o2.init_g(1)
    for loop in range(1, 3):
        o2.sweep(loop, 1)
        s = o2.state()
        assert s["err_fast_max"] <= 1e-6 + 1e-15
    assert s["positive_accept"] > 0 and s["negative_accept"] > 0


def test_boxmuller_fixed_order_arithmetic():
    """The Gaussian proposal's logarithm and cosine (include/pqmc_boxmuller.h,
    shared by the CUDA kernels and the oracle so that Gaussian jumps agree
    bit for bit) against the library functions: within 4 units in the last
    place over ran2 draws, the grid ends and the reduction boundaries of
    cos 2 pi t (1/8, 1/4, 3/8, 1/2, ...)."""
    import math
    from oracle.oracle import gauss_parts
    draws, _ = rng_draw(seed_words(7), 20000)
    u = draws.astype(np.float64)
    edges = np.array([2.0 ** -24, 1e-7, 0.125, 0.25, 0.375, 0.5, 0.625, 0.75, 0.875, 1.0 - 2.0 ** -24,
                      0.70710677, 0.70710683, 1.0], dtype=np.float32).astype(np.float64)
    u1 = np.concatenate([u[: u.size // 2], edges])
    u2 = np.concatenate([u[u.size // 2:], edges])
    out = gauss_parts(u1, u2)
    lg = np.array([math.log(x) for x in u1])
    cs = np.array([math.cos(2.0 * math.pi * x) for x in u2])
    jp = np.sqrt(-2.0 * lg) * cs
    ulp = np.spacing(1.0)
    assert np.all(np.abs(out[:, 0] - lg) <= 4 * ulp * np.maximum(np.abs(lg), 1e-300) + 1e-300)
    # the cosine: absolute error against an argument rounded to 2 pi * t
    assert np.all(np.abs(out[:, 1] - cs) <= 4 * ulp)
    assert np.all(np.abs(out[:, 2] - jp) <= 1e-14 * (1 + np.abs(jp)))
    assert np.all(out[u2 == 0.25, 1] == 0.0) and np.all(out[u2 == 0.5, 1] == -1.0) and out[-1, 1] == 1.0
