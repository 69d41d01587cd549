"""ctypes wrapper of the CPU oracle (oracle/pqmc_oracle.cpp).

TEST INFRASTRUCTURE ONLY -- imported by tests/, __graft_entry__.smoke() (to
check the GPU results) and bench.py's cpu_baseline leg.  Parity status: unpinned
against reference outputs (the reference has no golden vectors and cannot
be built here); see the header of pqmc_oracle.cpp for the invariants that
pin it instead.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from pqmc_allinone_gb300.abi import MeasStruct, ModelStruct, PqmcState
from pqmc_allinone_gb300.model import Model, record_width

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pqmc_oracle.cpp")
LIB = os.path.join(HERE, "_build", "liboracle.so")
_vp = ctypes.c_void_p
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no external libraries)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    hdrs = [os.path.join(HERE, "..", "include", h) for h in ("pqmc_gb300.h", "pqmc_boxmuller.h")]
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) > os.path.getmtime(SRC)
            and all(os.path.getmtime(LIB) > os.path.getmtime(h) for h in hdrs)):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB + ".tmp",
           SRC, "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB)
        for n in ("oracle_create",):
            getattr(L, n).argtypes = [ctypes.c_void_p, ctypes.POINTER(_vp)]
        L.oracle_time_parallel.restype = ctypes.c_double
        L.oracle_time_parallel.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_record_width.argtypes = [_vp]
        L.oracle_gauss_parts.argtypes = [_f64p, _f64p, ctypes.c_int, _f64p]
        _LIB = L
    return _LIB


def c128(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=np.complex128))


class OracleChain:
    """One chain on the CPU oracle, driven with the same calls as the GPU."""

    def __init__(self, m: Model, *, field: np.ndarray, seed_words=None, meas: bool | None = None,
                 proposal_kind: int | None = None):
        self.m = m
        self.L = lib()
        self.ms = ModelStruct(m, proposal_kind=proposal_kind)
        h = _vp()
        st = self.L.oracle_create(ctypes.cast(self.ms.ref, ctypes.c_void_p), ctypes.byref(h))
        assert st == 0, st
        self.h = h
        self.set_field(field)
        q, d = c128(m.slater_q), np.ascontiguousarray(m.slater_d, dtype=np.complex128)
        self._sq, self._sd = q, d
        self.L.oracle_set_slater(self.h, q.ctypes.data_as(_f64p), d.ctypes.data_as(_f64p))
        if seed_words is not None:
            self.set_rng(seed_words)
        self.meas = None
        if meas is None:
            meas = m.lat.dim == 2 and m.lat.n_sub == 2 and m.spec.bf_sets == 2
        if meas:
            self.meas = MeasStruct(m)
            self.L.oracle_set_meas_layout(self.h, self.meas.ref)

    def __del__(self):
        try:
            self.L.oracle_destroy(self.h)
        except Exception:
            pass

    # state
    def set_field(self, f):
        f = np.asfortranarray(f, dtype=np.float64)
        self.L.oracle_set_field(self.h, f.ctypes.data_as(_f64p))

    def field(self) -> np.ndarray:
        f = np.zeros((self.m.n_bf, self.m.ntime), order="F")
        self.L.oracle_get_field(self.h, f.ctypes.data_as(_f64p))
        return f

    def set_rng(self, words):
        w = (ctypes.c_int32 * 5)(*[int(x) for x in words])
        self.L.oracle_set_rng(self.h, w)

    def g(self) -> np.ndarray:
        g = np.zeros((self.m.ns, self.m.ns), dtype=np.complex128, order="F")
        self.L.oracle_get_g(self.h, g.ctypes.data_as(_f64p))
        return g

    def set_g(self, g):
        g = c128(g)
        self.L.oracle_set_g(self.h, g.ctypes.data_as(_f64p))

    def state(self) -> dict:
        s = PqmcState()
        self.L.oracle_get_state(self.h, ctypes.byref(s))
        return s.as_dict()

    def qd(self, blk: int):
        q = np.zeros((self.m.ns, self.m.nelec), dtype=np.complex128, order="F")
        d = np.zeros(self.m.nelec, dtype=np.complex128)
        self.L.oracle_get_qd(self.h, blk, q.ctypes.data_as(_f64p), d.ctypes.data_as(_f64p))
        return q, d

    def expkv(self):
        n = self.m.pdim ** 2 * self.m.max_pla * len(self.m.pf) * self.m.ntime
        a = np.zeros(n, dtype=np.complex128)
        b = np.zeros(n, dtype=np.complex128)
        self.L.oracle_get_expkv(self.h, a.ctypes.data_as(_f64p), b.ctypes.data_as(_f64p))
        return a, b

    # hot path
    def _ok(self, st, what):
        if st != 0:
            raise RuntimeError(f"oracle {what} -> {st}")

    def init_expkv(self):
        self._ok(self.L.oracle_init_expkv(self.h), "init_expkv")

    def init_g(self, start_time: int = 1):
        self._ok(self.L.oracle_init_g(self.h, start_time), "init_g")

    def update_phonon_field(self, pf_id: int, time: int):
        self._ok(self.L.oracle_update_phonon_field(self.h, pf_id, time), "update")

    def left_evolve_g(self, time, pf_id, two_way=True):
        self.L.oracle_left_evolve_g(self.h, time, pf_id, int(two_way))

    def right_evolve_g(self, time, pf_id, two_way=True):
        self.L.oracle_right_evolve_g(self.h, time, pf_id, int(two_way))

    def left_evolve(self, time, pf_id, mat):
        mat = c128(mat).copy(order="F")
        self.L.oracle_left_evolve(self.h, time, pf_id, mat.ctypes.data_as(_f64p), mat.shape[1])
        return mat

    def right_evolve(self, time, pf_id, mat):
        mat = c128(mat).copy(order="F")
        self.L.oracle_right_evolve(self.h, time, pf_id, mat.ctypes.data_as(_f64p), mat.shape[0])
        return mat

    def get_g_scratch(self, time, forward, loop=1):
        e = np.zeros(2)
        self._ok(self.L.oracle_get_g_scratch(self.h, time, int(forward), loop, e.ctypes.data_as(_f64p)),
                 "g_scratch")
        return e

    def cal_new_weight(self) -> complex:
        o = np.zeros(2)
        self._ok(self.L.oracle_cal_new_weight(self.h, o.ctypes.data_as(_f64p)), "new_weight")
        return complex(o[0], o[1])

    def take_measurement(self, time):
        self._ok(self.L.oracle_take_measurement(self.h, time), "take_measurement")

    def begin_measure(self, forward, time, meas_number=0):
        w = record_width(self.m)
        rec = np.zeros(w, dtype=np.complex128)
        done = ctypes.c_int(0)
        self._ok(self.L.oracle_begin_measure(self.h, int(forward), time, meas_number,
                                             rec.ctypes.data_as(_f64p), ctypes.byref(done)), "measure")
        return rec if done.value else None

    def sweep(self, first_loop, n_sweeps, warmup=1 << 30, meas_interval=1, meas_number=0, cap=0,
              max_slices=0):
        w = record_width(self.m)
        recs = np.zeros((max(cap, 1), w), dtype=np.complex128)
        n = ctypes.c_int(0)
        self._ok(self.L.oracle_sweep_ex(self.h, first_loop, n_sweeps, warmup, meas_interval,
                                        meas_number, recs.ctypes.data_as(_f64p), cap,
                                        ctypes.byref(n), max_slices), "sweep")
        return recs[: n.value]

    def time_parallel(self, n: int, threads: int, first_loop: int, max_slices: int) -> float:
        return self.L.oracle_time_parallel(self.h, n, threads, first_loop, max_slices)

    def expkv_single(self, kind, pf, pla, bf, inv):
        dim = self.m.pf[pf].dim
        out = np.zeros(dim * dim, dtype=np.complex128)
        self.L.oracle_expkv_single(self.h, kind, pf, pla, ctypes.c_double(bf), int(inv),
                                   out.ctypes.data_as(_f64p))
        return out.reshape((dim, dim), order="F")


def rng_draw(words, n):
    st = (ctypes.c_int32 * 5)(*[int(x) for x in words])
    out = (ctypes.c_float * n)()
    lib().oracle_rng_draw(st, n, out)
    return np.array(out[:], dtype=np.float32), list(st)


def gauss_parts(u1: np.ndarray, u2: np.ndarray) -> np.ndarray:
    """(log u1, cos 2 pi u2, Gaussian jump of width 1) per pair, by the
    fixed-order Box-Muller arithmetic the CUDA kernels share (n x 3)."""
    a = np.ascontiguousarray(u1, dtype=np.float64)
    b = np.ascontiguousarray(u2, dtype=np.float64)
    out = np.zeros((a.size, 3))
    lib().oracle_gauss_parts(a.ctypes.data_as(_f64p), b.ctypes.data_as(_f64p), a.size, out.ctypes.data_as(_f64p))
    return out
