"""Host mirror of the reference's Fortran hot-path interfaces on the GPU.

:class:`PqmcChain` exposes one method per reference subroutine, with the
reference's argument meaning (1-based ``time`` and ``pf_id``):

=========================  ===============================================
method                     reference
=========================  ===============================================
``init_expkv``             init_expKV + set_pf_expKV_mat
                           (src/mod_phonon_field.f90:423-450, 605-636)
``init_g(start_time)``     init_g_T0 (src/mod_evolution.f90:46-111)
``update_phonon_field``    update_phonon_field(ppf,time)
                           (src/mod_update.f90:13-201)
``left_evolve_g``          left_evolve(time,g_h,Ns,pf,.true.) (:236-285)
``right_evolve_g``         right_evolve(time,g_h,Ns,pf,.true.) (:287-328)
``left_evolve``            left_evolve(time,mat,n,pf,.false.)
``right_evolve``           right_evolve(time,mat,n,pf,.false.)
``get_g_scratch``          get_g_scratch_T0(time,forward,loop) (:113-195)
``cal_new_weight``         cal_new_weight_T0 (:359-408)
``take_measurement``       Meas_sys%take_measurement (mod_meas.f90:210)
``begin_measure``          Meas_sys%begin_measure (mod_meas.f90:729-763)
``sweep``                  the loop body of src/Main_PQMC.f90:81-156
=========================  ===============================================

Every call goes through the C-ABI of include/pqmc_gb300.h; a non-zero
status raises :class:`PqmcError` (the reference stops the program).
"""
from __future__ import annotations

import ctypes

import numpy as np

from .abi import MeasStruct, ModelStruct, PqmcError, PqmcState, check, global_struct, load_library
from .model import Model, record_width

_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)


def _c128(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=np.complex128))


class PqmcChain:
    """One Markov chain resident on the GPU."""

    def __init__(self, m: Model, *, field: np.ndarray, rng_words, meas: bool | None = None,
                 proposal_kind: int | None = None, handle: ctypes.c_void_p | None = None):
        self.m = m
        self.lib = load_library()
        self.ms = ModelStruct(m, proposal_kind=proposal_kind)
        self._owned = handle is None
        if handle is None:
            h = ctypes.c_void_p()
            self._chk(self.lib.pqmc_create(ctypes.byref(self.ms.s), ctypes.byref(h)), "pqmc_create")
            self.h = h
        else:
            self.h = handle
        self.set_field(field)
        q = _c128(m.slater_q)
        d = np.ascontiguousarray(m.slater_d, dtype=np.complex128)
        self._chk(self.lib.pqmc_set_slater(self.h, q.ctypes.data_as(_f64p), d.ctypes.data_as(_f64p)),
                  "pqmc_set_slater")
        self.set_rng(rng_words)
        self.meas = None
        if meas is None:
            meas = m.lat.dim == 2 and m.lat.n_sub == 2 and m.spec.bf_sets == 2
        if meas:
            self.meas = MeasStruct(m)
            self._chk(self.lib.pqmc_set_meas_layout(self.h, ctypes.byref(self.meas.s)),
                      "pqmc_set_meas_layout")

    def _chk(self, st, what):
        check(self.lib, st, what)

    def close(self):
        if getattr(self, "h", None) is not None and self._owned:
            self.lib.pqmc_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state -------------------------------------------------------
    def set_field(self, f):
        f = np.asfortranarray(f, dtype=np.float64)
        assert f.shape == (self.m.n_bf, self.m.ntime)
        self._chk(self.lib.pqmc_set_field(self.h, f.ctypes.data_as(_f64p)), "pqmc_set_field")

    def field(self) -> np.ndarray:
        f = np.zeros((self.m.n_bf, self.m.ntime), order="F")
        self._chk(self.lib.pqmc_get_field(self.h, f.ctypes.data_as(_f64p)), "pqmc_get_field")
        return f

    def set_field_slices(self, first_time: int, block):
        """boson_field(:, first_time..) from a host (n_bf, n) block; refreshes expKV there."""
        blk = np.asfortranarray(block, dtype=np.float64)
        assert blk.shape[0] == self.m.n_bf
        self._chk(self.lib.pqmc_set_field_slices(self.h, first_time, blk.shape[1], blk.ctypes.data_as(_f64p)),
                  "pqmc_set_field_slices")

    def get_field_slices(self, first_time: int, n: int, out=None) -> np.ndarray:
        if out is None:
            out = np.zeros((self.m.n_bf, n), order="F")
        self._chk(self.lib.pqmc_get_field_slices(self.h, first_time, n, out.ctypes.data_as(_f64p)),
                  "pqmc_get_field_slices")
        return out

    def set_rng(self, words):
        w = (ctypes.c_int32 * 5)(*[int(x) for x in words])
        self._chk(self.lib.pqmc_set_rng(self.h, w), "pqmc_set_rng")

    def g(self) -> np.ndarray:
        g = np.zeros((self.m.ns, self.m.ns), dtype=np.complex128, order="F")
        self._chk(self.lib.pqmc_get_g(self.h, g.ctypes.data_as(_f64p)), "pqmc_get_g")
        return g

    def set_g(self, g):
        g = _c128(g)
        self._chk(self.lib.pqmc_set_g(self.h, g.ctypes.data_as(_f64p)), "pqmc_set_g")

    def state(self) -> dict:
        s = PqmcState()
        self._chk(self.lib.pqmc_get_state(self.h, ctypes.byref(s)), "pqmc_get_state")
        return s.as_dict()

    # ---- global moves (update_global, mod_update.f90:250-467) -----------
    def set_global(self, gp: dict):
        """Global-move parameters (abi.global_params); pqmc_sweep then runs
        the driver's global step before every qualifying sweep."""
        s, keep = global_struct(gp)
        self._gkeep = keep
        self._chk(self.lib.pqmc_set_global(self.h, ctypes.byref(s)), "pqmc_set_global")

    def update_global(self, kind: int) -> bool:
        a = np.zeros(1, dtype=np.int32)
        self._chk(self.lib.pqmc_update_global(self.h, kind, a.ctypes.data_as(_i32p)), "update_global")
        return bool(a[0])

    def global_step(self, loop: int) -> int:
        a = np.zeros(1, dtype=np.int32)
        self._chk(self.lib.pqmc_global_step(self.h, loop, a.ctypes.data_as(_i32p)), "pqmc_global_step")
        return int(a[0])

    def global_counters(self) -> tuple[int, int]:
        a, r = ctypes.c_int64(0), ctypes.c_int64(0)
        self._chk(self.lib.pqmc_global_counters(self.h, ctypes.byref(a), ctypes.byref(r)), "pqmc_global_counters")
        return int(a.value), int(r.value)

    def set_state(self, st: dict):
        """Restore rng, accept counters and error maxima (a checkpoint's state())."""
        s = PqmcState.from_dict(st)
        self._chk(self.lib.pqmc_set_state(self.h, ctypes.byref(s)), "pqmc_set_state")

    def qd(self, blk: int):
        q = np.zeros((self.m.ns, self.m.nelec), dtype=np.complex128, order="F")
        d = np.zeros(self.m.nelec, dtype=np.complex128)
        self._chk(self.lib.pqmc_get_qd(self.h, blk, q.ctypes.data_as(_f64p), d.ctypes.data_as(_f64p)),
                  "pqmc_get_qd")
        return q, d

    # ---- hot path ------------------------------------------------------
    def init_expkv(self):
        self._chk(self.lib.pqmc_init_expkv(self.h), "init_expKV")

    def init_g(self, start_time: int = 1):
        self._chk(self.lib.pqmc_init_g(self.h, start_time), "init_g")

    # ---- finite temperature (src/mod_evolution.f90:409-785) -------------
    def set_temperature(self, proj: bool):
        """set_temperature: True for the projector path (the default), False
        for finite temperature; G is dropped, call init_g next."""
        self._chk(self.lib.pqmc_set_temperature(self.h, int(bool(proj))), "set_temperature")

    def proj(self) -> bool:
        v = ctypes.c_int(0)
        self._chk(self.lib.pqmc_get_temperature(self.h, ctypes.byref(v)), "get_temperature")
        return bool(v.value)

    def init_g_ft(self, start_time: int = 1):
        self._chk(self.lib.pqmc_init_g_ft(self.h, start_time), "init_g_FT")

    def get_g_scratch_ft(self, time: int, forward: bool, loop: int = 1) -> np.ndarray:
        e = np.zeros(2)
        self._chk(self.lib.pqmc_get_g_scratch_ft(self.h, time, int(forward), loop, e.ctypes.data_as(_f64p)),
                  "get_g_scratch_FT")
        return e

    def cal_new_weight_ft(self) -> complex:
        o = np.zeros(2)
        self._chk(self.lib.pqmc_cal_new_weight_ft(self.h, o.ctypes.data_as(_f64p)), "cal_new_weight_FT")
        return complex(o[0], o[1])

    def qdr_ft(self, blk: int):
        """(Q, D, R) of one block of the finite-temperature strings."""
        n = self.m.ns
        q = np.zeros((n, n), dtype=np.complex128, order="F")
        r = np.zeros((n, n), dtype=np.complex128, order="F")
        d = np.zeros(n, dtype=np.complex128)
        self._chk(self.lib.pqmc_get_qdr_ft(self.h, blk, q.ctypes.data_as(_f64p), d.ctypes.data_as(_f64p),
                                           r.ctypes.data_as(_f64p)), "get_qdr_FT")
        return q, d, r

    def update_phonon_field(self, pf_id: int, time: int):
        self._chk(self.lib.pqmc_update_phonon_field(self.h, pf_id, time), "update_phonon_field")

    def left_evolve_g(self, time: int, pf_id: int, two_way: bool = True):
        self._chk(self.lib.pqmc_left_evolve_g(self.h, time, pf_id, int(two_way)), "left_evolve")

    def right_evolve_g(self, time: int, pf_id: int, two_way: bool = True):
        self._chk(self.lib.pqmc_right_evolve_g(self.h, time, pf_id, int(two_way)), "right_evolve")

    def left_evolve(self, time: int, pf_id: int, mat) -> np.ndarray:
        mat = _c128(mat).copy(order="F")
        self._chk(self.lib.pqmc_left_evolve(self.h, time, pf_id, mat.ctypes.data_as(_f64p), mat.shape[1]),
                  "left_evolve")
        return mat

    def right_evolve(self, time: int, pf_id: int, mat) -> np.ndarray:
        mat = _c128(mat).copy(order="F")
        self._chk(self.lib.pqmc_right_evolve(self.h, time, pf_id, mat.ctypes.data_as(_f64p), mat.shape[0]),
                  "right_evolve")
        return mat

    def get_g_scratch(self, time: int, forward: bool, loop: int = 1) -> np.ndarray:
        e = np.zeros(2)
        self._chk(self.lib.pqmc_get_g_scratch(self.h, time, int(forward), loop, e.ctypes.data_as(_f64p)),
                  "get_g_scratch")
        return e

    def cal_new_weight(self) -> complex:
        o = np.zeros(2)
        self._chk(self.lib.pqmc_cal_new_weight(self.h, o.ctypes.data_as(_f64p)), "cal_new_weight")
        return complex(o[0], o[1])

    def set_field_device(self, ptr: int):
        """boson_field from a device pointer (n_bf, ntime) column-major."""
        self._chk(self.lib.pqmc_set_field_device(self.h, ctypes.c_void_p(ptr)), "pqmc_set_field_device")

    def logweight_grad_device(self, grad_ptr: int) -> complex:
        """Re log det(P^H B P) and its gradient (written to the device
        buffer at grad_ptr, (n_bf, ntime) doubles)."""
        o = np.zeros(2)
        self._chk(self.lib.pqmc_logweight_grad(self.h, o.ctypes.data_as(_f64p), ctypes.c_void_p(grad_ptr)),
                  "pqmc_logweight_grad")
        return complex(o[0], o[1])

    def sweep_slices(self, loop: int, first_tc: int, n_slices: int):
        """Slices first_tc .. first_tc+n_slices-1 of sweep `loop` (no measurement)."""
        self._chk(self.lib.pqmc_sweep_slices(self.h, loop, first_tc, n_slices), "pqmc_sweep_slices")

    def take_measurement(self, time: int):
        self._chk(self.lib.pqmc_take_measurement(self.h, time), "take_measurement")

    def begin_measure(self, forward: bool, time: int, meas_number: int = 0):
        rec = np.zeros(record_width(self.m), dtype=np.complex128)
        done = ctypes.c_int(0)
        self._chk(self.lib.pqmc_begin_measure(self.h, int(forward), time, meas_number,
                                              rec.ctypes.data_as(_f64p), ctypes.byref(done)),
                  "begin_measure")
        return rec if done.value else None

    def sweep(self, first_loop: int, n_sweeps: int = 1, *, warmup: int = 1 << 30, meas_interval: int = 1,
              meas_number: int = 0, cap: int = 0) -> np.ndarray:
        w = record_width(self.m)
        recs = np.zeros((max(cap, 1), w), dtype=np.complex128)
        n = ctypes.c_int(0)
        self._chk(self.lib.pqmc_sweep(self.h, first_loop, n_sweeps, warmup, meas_interval, meas_number,
                                      recs.ctypes.data_as(_f64p), cap, ctypes.byref(n)), "sweep")
        return recs[: n.value]


def global_generate(m: Model, gp: dict, kind: int, words, field):
    """pqmc_global_generate: the field of a global move on the host (no GPU).
    Returns (new field (n_bf, ntime), ph_ln_cw, t_first, t_last, rng words)."""
    lib = load_library()
    ms = ModelStruct(m)
    s, keep = global_struct(gp)
    f = np.array(field, dtype=np.float64, order="F", copy=True)
    w = np.array([int(x) for x in words], dtype=np.int32)
    ph = np.zeros(1)
    t = np.zeros(2, dtype=np.int32)
    check(lib, lib.pqmc_global_generate(ctypes.byref(ms.s), ctypes.byref(s), kind, w.ctypes.data_as(_i32p),
                                        f.ctypes.data_as(_f64p), ph.ctypes.data_as(_f64p),
                                        t[:1].ctypes.data_as(_i32p), t[1:].ctypes.data_as(_i32p)),
          "pqmc_global_generate")
    del keep
    return f, float(ph[0]), int(t[0]), int(t[1]), [int(x) for x in w]


def kernel_launches() -> int:
    return int(load_library().pqmc_kernel_launches())


__all__ = ["PqmcChain", "PqmcBatch", "PqmcError", "kernel_launches"]


class PqmcBatch:
    """Many chains advanced together (PQMC_PREC_FP64 or PQMC_PREC_MIXED).

    Each chain keeps the single-chain interface (``chains[i]``) for set-up,
    inspection and measurement; ``sweep(loop)`` advances every chain by one
    sweep of Main_PQMC.f90:99-154 (no measurement)."""

    def __init__(self, models, fields, rng_words, *, precision: int = 1, meas: bool | None = False):
        self.lib = load_library()
        self.models = list(models)
        self._ms = [ModelStruct(m) for m in self.models]
        arr = (ctypes.POINTER(type(self._ms[0].s)) * len(self._ms))(
            *[ctypes.pointer(x.s) for x in self._ms])
        h = ctypes.c_void_p()
        check(self.lib, self.lib.pqmc_batch_create(arr, len(self._ms), precision, ctypes.byref(h)),
              "pqmc_batch_create")
        self.h = h
        self.chains = []
        for i, (m, f, w) in enumerate(zip(self.models, fields, rng_words)):
            ch = ctypes.c_void_p()
            check(self.lib, self.lib.pqmc_batch_chain(self.h, i, ctypes.byref(ch)), "pqmc_batch_chain")
            self.chains.append(PqmcChain(m, field=f, rng_words=w, meas=meas, handle=ch))

    def init(self):
        """init_expKV + init_g_T0(1) of every chain (batched for mixed batches)."""
        check(self.lib, self.lib.pqmc_batch_init(self.h), "pqmc_batch_init")

    def sweep(self, loop: int):
        check(self.lib, self.lib.pqmc_batch_sweep(self.h, loop), "pqmc_batch_sweep")

    def sweep_slices(self, loop: int, first_tc: int, n_slices: int):
        """Slices first_tc .. first_tc+n_slices-1 of sweep `loop` of every chain."""
        check(self.lib, self.lib.pqmc_batch_sweep_slices(self.h, loop, first_tc, n_slices),
              "pqmc_batch_sweep_slices")

    def stream(self) -> int:
        """The cudaStream_t (as an integer) the batched kernels run on."""
        s = ctypes.c_void_p()
        check(self.lib, self.lib.pqmc_batch_stream(self.h, ctypes.byref(s)), "pqmc_batch_stream")
        return int(s.value or 0)

    def info(self) -> dict:
        v = np.zeros(5, dtype=np.int32)
        check(self.lib, self.lib.pqmc_batch_info(self.h, v.ctypes.data_as(_i32p)), "pqmc_batch_info")
        return {"chains": int(v[0]), "groups": int(v[1]), "delay_depth": int(v[2]),
                "flush": {2: "exact", 1: "tcgen05"}.get(int(v[3]), "mma.sync"), "precision": int(v[4])}

    PHASES = ("prep", "scan", "flush", "wrap", "recompute", "split")

    def set_timing(self, enable: bool):
        check(self.lib, self.lib.pqmc_batch_set_timing(self.h, 1 if enable else 0), "pqmc_batch_set_timing")

    def timing(self) -> dict:
        """{phase: (total ms, timed launches)} since set_timing(True)."""
        ms = np.zeros(len(self.PHASES))
        n = (ctypes.c_longlong * len(self.PHASES))()
        check(self.lib, self.lib.pqmc_batch_get_timing(self.h, ms.ctypes.data_as(_f64p), n),
              "pqmc_batch_get_timing")
        return {p: (float(ms[i]), int(n[i])) for i, p in enumerate(self.PHASES)}

    def flush_rounds(self) -> list:
        """Per chain: flushes with panel columns since set_timing (G read-modify-writes)."""
        n = (ctypes.c_longlong * len(self.chains))()
        check(self.lib, self.lib.pqmc_batch_flush_rounds(self.h, n), "pqmc_batch_flush_rounds")
        return [int(v) for v in n]

    def scan_profile(self) -> list:
        """Per chain since set_timing(True): (scan SM cycles, accepted moves,
        rejected proposals) of its sequential scan."""
        n = (ctypes.c_longlong * (3 * len(self.chains)))()
        check(self.lib, self.lib.pqmc_batch_scan_profile(self.h, n), "pqmc_batch_scan_profile")
        return [(int(n[3 * i]), int(n[3 * i + 1]), int(n[3 * i + 2])) for i in range(len(self.chains))]

    def set_delay(self, depth: int):
        check(self.lib, self.lib.pqmc_batch_set_delay(self.h, depth), "pqmc_batch_set_delay")

    def autotune(self, loop: int, first_tc: int, n_slices: int, candidates=(32, 48, 64, 96, 128)):
        """Delay-depth autotuner: one block of n_slices per candidate from
        (loop, first_tc) on (genuine Monte Carlo steps); keeps the fastest.
        Returns (best depth, {depth: ms per slice})."""
        cand = np.ascontiguousarray(candidates, dtype=np.int32)
        ms = np.zeros(len(cand))
        best = np.zeros(1, dtype=np.int32)
        check(self.lib, self.lib.pqmc_batch_autotune(self.h, loop, first_tc, n_slices, cand.ctypes.data_as(_i32p),
                                                      len(cand), best.ctypes.data_as(_i32p),
                                                      ms.ctypes.data_as(_f64p)), "pqmc_batch_autotune")
        return int(best[0]), {int(k): float(v) for k, v in zip(cand, ms)}

    WRAP_TILES = {0: "gathered blocks", 1: "1 column item per CTA", 2: "2 column items per CTA"}

    def set_wrap_tile(self, ci: int):
        """Tile shape of the two-way wrap: 1 or 2 column items per staged CTA,
        0 for the gathered form (bit-identical results in every shape)."""
        check(self.lib, self.lib.pqmc_batch_set_wrap_tile(self.h, ci), "pqmc_batch_set_wrap_tile")

    def wrap_tile(self) -> int:
        v = ctypes.c_int(0)
        check(self.lib, self.lib.pqmc_batch_get_wrap_tile(self.h, ctypes.byref(v)), "pqmc_batch_get_wrap_tile")
        return int(v.value)

    def set_flush_tile(self, ct: int):
        """Flush of the exact round update: 64 or 32 columns of G per CTA, or
        the pipeline with 2 or 1 CTAs per row tile."""
        check(self.lib, self.lib.pqmc_batch_set_flush_tile(self.h, ct), "pqmc_batch_set_flush_tile")

    def flush_tile(self) -> int:
        v = ctypes.c_int(0)
        check(self.lib, self.lib.pqmc_batch_get_flush_tile(self.h, ctypes.byref(v)), "pqmc_batch_get_flush_tile")
        return int(v.value)

    def set_gemm_engine(self, engine: int):
        """Engine of the recompute's GEMMs: 0 double-float on the FP32 pipe,
        1 Ozaki-split BF16 on the tensor cores."""
        check(self.lib, self.lib.pqmc_batch_set_gemm_engine(self.h, engine), "pqmc_batch_set_gemm_engine")

    def gemm_engine(self) -> int:
        v = ctypes.c_int(0)
        check(self.lib, self.lib.pqmc_batch_get_gemm_engine(self.h, ctypes.byref(v)), "pqmc_batch_get_gemm_engine")
        return int(v.value)

    def set_scan_chunk(self, qc: int):
        """Panel columns per streamed chunk of the scan (1 .. the largest that fits)."""
        check(self.lib, self.lib.pqmc_batch_set_scan_chunk(self.h, qc), "pqmc_batch_set_scan_chunk")

    def scan_chunk(self, with_max: bool = False):
        """The scan's panel chunk (and, with_max, the largest that fits)."""
        v, mx = ctypes.c_int(0), ctypes.c_int(0)
        check(self.lib, self.lib.pqmc_batch_get_scan_chunk(self.h, ctypes.byref(v), ctypes.byref(mx)),
              "pqmc_batch_get_scan_chunk")
        return (int(v.value), int(mx.value)) if with_max else int(v.value)

    TILE_FLUSH = (64, 32, 2, 1)

    @staticmethod
    def flush_tile_name(ct: int) -> str:
        return f"{ct} columns per CTA" if ct in (64, 32) else f"pipeline, {ct} CTA(s) per row tile"

    @staticmethod
    def scan_chunk_candidates(qc_max: int):
        """The scan chunks the tile autotuner times, in its ms_out order."""
        return (qc_max, (3 * qc_max + 3) // 4, (qc_max + 1) // 2)

    def autotune_tiles(self, loop: int, first_tc: int, n_slices: int):
        """Tile-shape autotuner at the current delay depth: every wrap tile,
        then (exact round update) every flush tile, then every scan chunk,
        each timed over n_slices slices from (loop, first_tc); keeps the
        fastest of each.  Returns ((best wrap tile, best flush tile, best
        scan chunk), {wrap tile: ms}, {flush tile: ms}, {scan chunk: ms})
        with None where a shape does not fit or does not apply."""
        ms = np.zeros(10)
        best = (ctypes.c_int * 3)()
        _, qmax = self.scan_chunk(with_max=True)
        check(self.lib, self.lib.pqmc_batch_autotune_tiles(self.h, loop, first_tc, n_slices, best,
                                                            ms.ctypes.data_as(_f64p)), "pqmc_batch_autotune_tiles")
        val = [float(v) if v >= 0 else None for v in ms]
        # the scan slots as a list of (chunk, ms): two slots can hold the same chunk when qc_max is small
        scan = list(zip(self.scan_chunk_candidates(qmax), val[7:10]))
        return ((int(best[0]), int(best[1]), int(best[2])), dict(zip((0, 1, 2), val[:3])),
                dict(zip(self.TILE_FLUSH, val[3:7])), scan)

    def tiles_timed(self, wrap_table: dict, flush_table: dict, scan_slots: list) -> int:
        """Blocks of slices an autotune_tiles call ran: every wrap and scan
        chunk slot, and the flush slots with the exact round update."""
        return len(wrap_table) + sum(v is not None for v in flush_table.values()) + len(scan_slots)

    def set_measure(self, warmup: int, meas_interval: int = 1, meas_number: int = 0):
        """Equal-time measurements in batched sweeps (chains built with meas=True)."""
        check(self.lib, self.lib.pqmc_batch_set_measure(self.h, warmup, meas_interval, meas_number),
              "pqmc_batch_set_measure")

    def records(self, i: int, cap: int = 1024) -> np.ndarray:
        """Finished measurement records of chain i, complex (n, width)."""
        w = record_width(self.models[i])
        out = np.zeros((cap, 2 * w))
        n = np.zeros(1, dtype=np.int32)
        check(self.lib, self.lib.pqmc_batch_records(self.h, i, out.ctypes.data_as(_f64p), cap,
                                                     n.ctypes.data_as(_i32p)), "pqmc_batch_records")
        return out[:n[0]].view(np.complex128)

    def set_graphs(self, enable: bool):
        """Replay each slice's family steps from a captured CUDA graph."""
        check(self.lib, self.lib.pqmc_batch_set_graphs(self.h, 1 if enable else 0), "pqmc_batch_set_graphs")

    def field_slices(self, first_time: int, n: int, host, to_device: bool):
        """Slices first_time..first_time+n-1 of every chain's field, host
        blocks chain after chain ((n_bf, n) column-major each, clipped to
        each chain's ntime), in one call (pinned host memory: host may be a
        numpy view of a pinned buffer)."""
        check(self.lib, self.lib.pqmc_batch_field_slices(self.h, first_time, n,
                                                          host.ctypes.data_as(_f64p), 1 if to_device else 0),
              "pqmc_batch_field_slices")

    def states(self) -> list:
        """state() of every chain with one wait."""
        arr = (PqmcState * len(self.chains))()
        check(self.lib, self.lib.pqmc_batch_states(self.h, arr), "pqmc_batch_states")
        return [a.as_dict() for a in arr]

    def classes(self) -> list:
        """Geometry classes of the batch: [{chains, ns, ntime, delay_depth, flush, groups}]."""
        n = np.zeros(1, dtype=np.int32)
        check(self.lib, self.lib.pqmc_batch_classes(self.h, n.ctypes.data_as(_i32p)), "pqmc_batch_classes")
        out = []
        for k in range(int(n[0])):
            v = np.zeros(6, dtype=np.int32)
            check(self.lib, self.lib.pqmc_batch_class_info(self.h, k, v.ctypes.data_as(_i32p)),
                  "pqmc_batch_class_info")
            out.append({"chains": int(v[0]), "ns": int(v[1]), "ntime": int(v[2]), "delay_depth": int(v[3]),
                        "flush": {2: "exact", 1: "tcgen05"}.get(int(v[4]), "mma.sync"), "groups": int(v[5])})
        return out

    def graph_count(self) -> int:
        n = np.zeros(1, dtype=np.int32)
        check(self.lib, self.lib.pqmc_batch_graph_count(self.h, n.ctypes.data_as(_i32p)), "pqmc_batch_graph_count")
        return int(n[0])

    def set_flush(self, mode: int):
        """2: exact round update (default; double-float Woodbury update of the
        round from G with Ozaki-split tcgen05 products, double-float wraps),
        1: tcgen05 flush of the scan's FP32 panels, 0: mma.sync flush of them
        (both delay depth <= 64 on the tensor cores)."""
        check(self.lib, self.lib.pqmc_batch_set_flush(self.h, mode), "pqmc_batch_set_flush")

    def close(self):
        if getattr(self, "h", None) is not None:
            for c in self.chains:
                c.h = None
            self.lib.pqmc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def recompute_gemm_check(ta: str, tb: str, a: np.ndarray, b: np.ndarray, engine: int) -> np.ndarray:
    """The recompute's batched GEMM on host operands (validation):
    C_i = op(A_i) op(B_i) for a (count, rows, cols) stack of each, op 'N' or
    'C' (conjugate transpose); engine 0 (double-float, FP32 pipe) or 1
    (Ozaki, tensor cores).  Returns C (count, m, n)."""
    lib = load_library()
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    count = a.shape[0]
    m = a.shape[2] if ta == "C" else a.shape[1]
    k = a.shape[1] if ta == "C" else a.shape[2]
    n = b.shape[1] if tb == "C" else b.shape[2]
    af = np.ascontiguousarray(a.transpose(0, 2, 1))   # column-major per matrix
    bf = np.ascontiguousarray(b.transpose(0, 2, 1))
    cf = np.zeros((count, n, m), dtype=np.complex128)
    check(lib, lib.pqmc_recompute_gemm_check(ta.encode(), tb.encode(), m, n, k, count,
                                              af.view(np.float64).ctypes.data_as(_f64p), a.shape[1],
                                              bf.view(np.float64).ctypes.data_as(_f64p), b.shape[1],
                                              cf.view(np.float64).ctypes.data_as(_f64p), m, int(engine)),
          "pqmc_recompute_gemm_check")
    return cf.transpose(0, 2, 1)


def exact_update_check(g: np.ndarray, sites, delta, flush_tile: int = 64) -> np.ndarray:
    """The batch's exact round update applied to a host G (validation):
    returns G + G(:,S) Delta_S W^-1 (E_S - G(S,:)), sites in acceptance
    order (dim per move), delta (n_moves, dim, dim); flush_tile 64
    (k_xgemm<1>), 32 (k_xflush2), or 2 / 1 (the pipeline k_xflushp)."""
    lib = load_library()
    ns = g.shape[0]
    d = np.asarray(delta, dtype=np.complex128)
    nb, dim = d.shape[0], d.shape[1]
    s = np.ascontiguousarray(sites, dtype=np.int32)
    gg = np.asfortranarray(g, dtype=np.complex128).copy(order="F")
    dl = np.ascontiguousarray(np.stack([np.asfortranarray(x).ravel(order="F") for x in d]))
    check(lib, lib.pqmc_exact_update_check_tile(ns, len(s), dim, s.ctypes.data_as(_i32p),
                                                 dl.view(np.float64).ctypes.data_as(_f64p),
                                                 gg.ravel(order="K").view(np.float64).ctypes.data_as(_f64p),
                                                 int(flush_tile)),
          "pqmc_exact_update_check")
    return gg
