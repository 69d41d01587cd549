"""The allocation-free recompute entry point against the chain's own and the oracle.

pqmc_cal_g_and_det_noalloc serves callers that cannot call cudaMalloc: hosts
that hand the whole device to a fixed memory arena at start-up, and Fortran
drivers whose only CUDA binding is this C library.  It keeps its work space
in a fixed device array inside the library.  This test feeds it the
stabilised factors of a chain after init_g_T0 and checks G and the
log-weight against what pqmc_init_g produced and G against the CPU oracle's
init_g_T0 on the same field, on two calls in a row (the shared work space
must not leak state between calls).  It runs last in the suite and also
passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tests.helpers import SEED_WORDS, epsocz_small, rel_fro

pytestmark = pytest.mark.gpu

G_TOL = 1e-10   # relative Frobenius, as in the other GPU parity tests


def _dev(torch, a):
    """Complex column-major numpy array -> float64 CUDA tensor with the same bytes."""
    flat = np.asfortranarray(a, dtype=np.complex128).ravel(order="F").view(np.float64)
    return torch.from_numpy(flat.copy()).to("cuda")


def test_noalloc_recompute_matches_init_g():
    torch = pytest.importorskip("torch")
    from pqmc_allinone_gb300.engine import PqmcChain
    m, f = epsocz_small(L=4, ntime=40, ngroup=10, lam=0.8, alpha=0.3)
    ch = PqmcChain(m, field=f, rng_words=SEED_WORDS)
    ch.init_expkv()
    ch.init_g(1)
    g_ref = ch.g()
    from oracle.oracle import OracleChain
    o = OracleChain(m, field=f, seed_words=SEED_WORDS)
    o.init_expkv()
    o.init_g(1)
    g_oracle = o.g()
    lncw = ch.state()["ln_cw"]
    ql, _ = ch.qd(m.nblock)          # left factor X = Q_string(nblock), L = X^H
    qr, _ = ch.qd(m.nblock - 1)      # right factor after the last stabilisation
    sumlogd = sum(np.log(ch.qd(b)[1]).sum() for b in range(1, m.nblock + 1))
    x_d, r_d = _dev(torch, ql), _dev(torch, qr)
    lib = ch.lib
    fn = lib.pqmc_cal_g_and_det_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    for call in range(2):
        g_d = torch.full((2 * m.ns * m.ns,), float("nan"), dtype=torch.float64, device="cuda")
        ld_d = torch.zeros(2, dtype=torch.float64, device="cuda")
        st = fn(x_d.data_ptr(), r_d.data_ptr(), m.ns, m.nelec, g_d.data_ptr(), ld_d.data_ptr(), None)
        assert st == 0, lib.pqmc_last_error()
        g = g_d.cpu().numpy().view(np.complex128).reshape((m.ns, m.ns), order="F")
        assert rel_fro(g, g_ref) < G_TOL, call
        assert rel_fro(g, g_oracle) < G_TOL, call
        ld = complex(*ld_d.cpu().numpy())
        assert abs((ld + sumlogd).real - lncw.real) <= 1e-9 * abs(lncw.real) + 1e-9, call


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    from pqmc_allinone_gb300.abi import load_library
    lib = load_library()
    fn = lib.pqmc_cal_g_and_det_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    assert fn(p, p, 513, 8, p, p, None) == 1
    assert fn(p, p, 600, 300, p, p, None) == 1
    assert b"ns=" in lib.pqmc_last_error()


def test_noalloc_refuses_stream_capture():
    """The call reads its pivot flag back and synchronises, which a CUDA-graph
    capture does not allow: on a capturing stream it returns PQMC_ERR_ARG
    before touching the GPU, and the capture (here of one other kernel)
    stays valid and replays."""
    torch = pytest.importorskip("torch")
    from pqmc_allinone_gb300.abi import load_library
    lib = load_library()
    fn = lib.pqmc_cal_g_and_det_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    cnt = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    cnt.add_(0.0)   # the add kernel loaded before the capture
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        st = fn(p, p, 8, 4, p, p, ctypes.c_void_p(s.cuda_stream))
        cnt.add_(1.0)
    assert st == 1
    assert b"captured" in lib.pqmc_last_error()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert float(cnt[0]) == 2.0
