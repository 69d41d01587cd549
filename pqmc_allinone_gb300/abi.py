"""ctypes view of include/pqmc_gb300.h and the loader of the CUDA library.

The loader fails loudly: there is no CPU fallback for the hot path.  The
library is built in-tree (``pqmc_allinone_gb300/_build/libpqmc_gb300.so``)
by :mod:`pqmc_allinone_gb300.build`.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .model import Model, meas_tables

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpqmc_gb300.so")

PQMC_OK = 0
ERRORS = {1: "PQMC_ERR_ARG", 2: "PQMC_ERR_CUDA", 3: "PQMC_ERR_SINGULAR", 4: "PQMC_ERR_TIMEOUT",
          5: "PQMC_ERR_STATE", 6: "PQMC_ERR_NOMEM"}
N_SCALAR, N_FIELD = 3, 25
PREC_FP64, PREC_MIXED = 0, 1

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)


class PqmcModel(ctypes.Structure):
    _fields_ = [
        ("ns", ctypes.c_int32), ("nelec", ctypes.c_int32), ("ntime", ctypes.c_int32),
        ("ngroup", ctypes.c_int32), ("n_pf", ctypes.c_int32), ("max_dim", ctypes.c_int32),
        ("max_pla", ctypes.c_int32), ("n_bf", ctypes.c_int32), ("expkv_kind", ctypes.c_int32),
        ("ncopy", ctypes.c_int32), ("tr_weight", ctypes.c_int32), ("metropolis", ctypes.c_int32),
        ("greatest_decent", ctypes.c_int32), ("local_update", ctypes.c_int32),
        ("proposal_kind", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("delt", ctypes.c_double), ("mass", ctypes.c_double), ("stiff", ctypes.c_double),
        ("biased_phonon", ctypes.c_double), ("jump_distance", ctypes.c_double),
        ("pf_dim", _i32p), ("pf_npla", _i32p), ("pf_k_exist", _i32p), ("pf_v_exist", _i32p),
        ("pf_k_coe", _f64p), ("pf_v_coe", _f64p), ("pf_kmat", _f64p), ("pf_vmat", _f64p),
        ("pla_site_list", _i32p), ("bf_list", _i32p), ("boundary_crossing", _i32p),
        ("bc_phases", _f64p),
    ]


class PqmcMeasLayout(ctypes.Structure):
    _fields_ = [
        ("n_cell", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("cell_sites", _i32p), ("cell_bf", _i32p), ("cell_xnb", _i32p), ("cell_ynb", _i32p),
        ("cell_cross", _i32p), ("rel_index", _i32p), ("bc_phase", _f64p), ("k_phase", _f64p),
        ("hop", ctypes.c_double), ("ep_parameter", ctypes.c_double),
    ]


class PqmcState(ctypes.Structure):
    _fields_ = [
        ("ln_cw", ctypes.c_double * 2), ("err_fast_max", ctypes.c_double),
        ("err_fast", ctypes.c_double), ("positive_accept", ctypes.c_int64),
        ("negative_accept", ctypes.c_int64), ("rng", ctypes.c_int32 * 5),
        ("reserved", ctypes.c_int32), ("err_g", ctypes.c_double), ("err_g_rel_max", ctypes.c_double),
    ]

    @classmethod
    def from_dict(cls, d: dict) -> "PqmcState":
        s = cls()
        s.ln_cw[0], s.ln_cw[1] = complex(d.get("ln_cw", 0)).real, complex(d.get("ln_cw", 0)).imag
        s.err_fast_max, s.err_fast = float(d["err_fast_max"]), float(d["err_fast"])
        s.positive_accept, s.negative_accept = int(d["positive_accept"]), int(d["negative_accept"])
        for k in range(5):
            s.rng[k] = int(d["rng"][k])
        s.err_g, s.err_g_rel_max = float(d["err_g"]), float(d["err_g_rel_max"])
        return s

    def as_dict(self) -> dict:
        return dict(ln_cw=complex(self.ln_cw[0], self.ln_cw[1]), err_fast_max=self.err_fast_max,
                    err_fast=self.err_fast, positive_accept=self.positive_accept,
                    negative_accept=self.negative_accept, rng=list(self.rng), err_g=self.err_g,
                    err_g_rel_max=self.err_g_rel_max)


class GlobalParams(ctypes.Structure):
    """pqmc_global_params (global moves, src/mod_update.f90:250-467)."""
    _fields_ = [
        ("n_global_update", ctypes.c_int32), ("global_update_loop", ctypes.c_int32),
        ("flip", ctypes.c_int32), ("shift", ctypes.c_int32), ("rotate", ctypes.c_int32),
        ("lat_dim", ctypes.c_int32), ("n_cell", ctypes.c_int32), ("bf_sets", ctypes.c_int32),
        ("distance", ctypes.c_double), ("cell_rpos", ctypes.POINTER(ctypes.c_double)),
    ]


def global_params(m: Model, *, global_update_distance: float = 1.0, n_global_update: int = 1,
                  global_update_loop: int = 2, flip: bool = False, shift: bool = False,
                  rotate: bool | None = None) -> dict:
    """The global-update namelist values of input.f90:19-22,71-75 for model m
    (distance scaled by char_length as in input.f90:184; the "rotate" move
    for EPSOCZ models as in Main_PQMC.f90:92)."""
    if rotate is None:
        rotate = m.spec.model_name.strip() == "EPSOCZ"
    return {"n_global_update": int(n_global_update), "global_update_loop": int(global_update_loop),
            "flip": int(flip), "shift": int(shift), "rotate": int(rotate), "lat_dim": int(m.lat.dim),
            "n_cell": int(m.lat.n_cell), "bf_sets": int(m.spec.bf_sets),
            "distance": float(global_update_distance) * float(m.char_length),
            "cell_rpos": np.ascontiguousarray(m.lat.cell_rpos, dtype=np.float64)}


def global_struct(gp: dict):
    """(ctypes struct, kept buffers) of a global_params dict."""
    rpos = np.ascontiguousarray(gp["cell_rpos"], dtype=np.float64)   # (n_cell, dim) == Fortran (dim, n_cell)
    s = GlobalParams(gp["n_global_update"], gp["global_update_loop"], gp["flip"], gp["shift"], gp["rotate"],
                     gp["lat_dim"], gp["n_cell"], gp["bf_sets"], gp["distance"],
                     rpos.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return s, rpos


def _ptr(a: np.ndarray, ty):
    return a.ctypes.data_as(ty)


class ModelStruct:
    """A filled ``pqmc_model`` plus the numpy buffers it points into."""

    def __init__(self, m: Model, *, proposal_kind: int | None = None):
        spec = m.spec
        npf = len(m.pf)
        fl = m.flat_tables()
        self.keep = dict(
            pf_dim=np.array([t.dim for t in m.pf], dtype=np.int32),
            pf_npla=np.array([t.n_pla for t in m.pf], dtype=np.int32),
            pf_k_exist=np.array([int(p.k_exist) for p in spec.pfs], dtype=np.int32),
            pf_v_exist=np.array([int(p.v_exist) for p in spec.pfs], dtype=np.int32),
            pf_k_coe=np.ascontiguousarray(m.k_coe.astype(np.complex128)),
            pf_v_coe=np.ascontiguousarray(m.v_coe.astype(np.complex128)),
            pf_kmat=fl["kmat"], pf_vmat=fl["vmat"], pla_site_list=fl["pla_site_list"],
            bf_list=fl["bf_list"], boundary_crossing=fl["boundary_crossing"],
            bc_phases=fl["bc_phases"],
        )
        k = self.keep
        self.s = PqmcModel(
            ns=m.ns, nelec=m.nelec, ntime=m.ntime, ngroup=m.ngroup, n_pf=npf, max_dim=m.pdim,
            max_pla=m.max_pla, n_bf=m.n_bf, expkv_kind=m.expkv_kind, ncopy=spec.ncopy,
            tr_weight=int(spec.tr_weight), metropolis=int(spec.metropolis),
            greatest_decent=int(spec.greatest_decent), local_update=int(spec.local_update),
            proposal_kind=spec.proposal_kind if proposal_kind is None else proposal_kind, reserved=0,
            delt=spec.delt, mass=m.M, stiff=m.D, biased_phonon=spec.biased_phonon,
            jump_distance=m.jump_distance,
            pf_dim=_ptr(k["pf_dim"], _i32p), pf_npla=_ptr(k["pf_npla"], _i32p),
            pf_k_exist=_ptr(k["pf_k_exist"], _i32p), pf_v_exist=_ptr(k["pf_v_exist"], _i32p),
            pf_k_coe=_ptr(k["pf_k_coe"], _f64p), pf_v_coe=_ptr(k["pf_v_coe"], _f64p),
            pf_kmat=_ptr(k["pf_kmat"], _f64p), pf_vmat=_ptr(k["pf_vmat"], _f64p),
            pla_site_list=_ptr(k["pla_site_list"], _i32p), bf_list=_ptr(k["bf_list"], _i32p),
            boundary_crossing=_ptr(k["boundary_crossing"], _i32p),
            bc_phases=_ptr(k["bc_phases"], _f64p),
        )

    @property
    def ref(self):
        return ctypes.byref(self.s)


class MeasStruct:
    def __init__(self, m: Model):
        t = meas_tables(m)
        self.keep = {k: np.ascontiguousarray(v) for k, v in t.items()}
        k = self.keep
        self.s = PqmcMeasLayout(
            n_cell=m.lat.n_cell, reserved=0,
            cell_sites=_ptr(k["cell_sites"], _i32p), cell_bf=_ptr(k["cell_bf"], _i32p),
            cell_xnb=_ptr(k["cell_xnb"], _i32p), cell_ynb=_ptr(k["cell_ynb"], _i32p),
            cell_cross=_ptr(k["cell_cross"], _i32p), rel_index=_ptr(k["rel_index"], _i32p),
            bc_phase=_ptr(k["bc_phase"], _f64p), k_phase=_ptr(k["k_phase"], _f64p),
            hop=m.spec.hop, ep_parameter=m.spec.ep_parameter,
        )

    @property
    def ref(self):
        return ctypes.byref(self.s)


_LIB = None


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load libpqmc_gb300.so; raises if it is missing (no CPU fallback)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"pqmc CUDA library not built: {p} is missing; run "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    sigs = {
        "pqmc_create": ([ctypes.POINTER(PqmcModel), ctypes.POINTER(vp)], ctypes.c_int),
        "pqmc_destroy": ([vp], ctypes.c_int),
        "pqmc_set_meas_layout": ([vp, ctypes.POINTER(PqmcMeasLayout)], ctypes.c_int),
        "pqmc_set_field": ([vp, _f64p], ctypes.c_int),
        "pqmc_get_field": ([vp, _f64p], ctypes.c_int),
        "pqmc_set_slater": ([vp, _f64p, _f64p], ctypes.c_int),
        "pqmc_get_g": ([vp, _f64p], ctypes.c_int),
        "pqmc_set_g": ([vp, _f64p], ctypes.c_int),
        "pqmc_get_state": ([vp, ctypes.POINTER(PqmcState)], ctypes.c_int),
        "pqmc_set_rng": ([vp, _i32p], ctypes.c_int),
        "pqmc_set_state": ([vp, ctypes.POINTER(PqmcState)], ctypes.c_int),
        "pqmc_global_generate": ([ctypes.POINTER(PqmcModel), ctypes.POINTER(GlobalParams), ctypes.c_int, _i32p,
                                  _f64p, _f64p, _i32p, _i32p], ctypes.c_int),
        "pqmc_set_global": ([vp, ctypes.POINTER(GlobalParams)], ctypes.c_int),
        "pqmc_update_global": ([vp, ctypes.c_int, _i32p], ctypes.c_int),
        "pqmc_global_step": ([vp, ctypes.c_int, _i32p], ctypes.c_int),
        "pqmc_global_counters": ([vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
                                 ctypes.c_int),
        "pqmc_get_qd": ([vp, ctypes.c_int, _f64p, _f64p], ctypes.c_int),
        "pqmc_init_expkv": ([vp], ctypes.c_int),
        "pqmc_init_g": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_update_phonon_field": ([vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "pqmc_left_evolve_g": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "pqmc_right_evolve_g": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "pqmc_left_evolve": ([vp, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int], ctypes.c_int),
        "pqmc_right_evolve": ([vp, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int], ctypes.c_int),
        "pqmc_get_g_scratch": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p], ctypes.c_int),
        "pqmc_cal_new_weight": ([vp, _f64p], ctypes.c_int),
        "pqmc_set_temperature": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_get_temperature": ([vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pqmc_init_g_ft": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_get_g_scratch_ft": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p], ctypes.c_int),
        "pqmc_cal_new_weight_ft": ([vp, _f64p], ctypes.c_int),
        "pqmc_get_qdr_ft": ([vp, ctypes.c_int, _f64p, _f64p, _f64p], ctypes.c_int),
        "pqmc_take_measurement": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_begin_measure": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p,
                                ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pqmc_sweep": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                        _f64p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pqmc_set_field_device": ([vp, ctypes.c_void_p], ctypes.c_int),
        "pqmc_logweight_grad": ([vp, _f64p, ctypes.c_void_p], ctypes.c_int),
        "pqmc_batch_create": ([ctypes.POINTER(ctypes.POINTER(PqmcModel)), ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(vp)], ctypes.c_int),
        "pqmc_batch_destroy": ([vp], ctypes.c_int),
        "pqmc_batch_chain": ([vp, ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
        "pqmc_batch_sweep": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_set_delay": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_set_flush": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_set_measure": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_records": ([vp, ctypes.c_int, _f64p, ctypes.c_int, _i32p], ctypes.c_int),
        "pqmc_batch_autotune": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, ctypes.c_int, _i32p, _f64p],
                                ctypes.c_int),
        "pqmc_batch_set_wrap_tile": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_get_wrap_tile": ([vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pqmc_batch_autotune_tiles": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _f64p],
                                      ctypes.c_int),
        "pqmc_batch_set_flush_tile": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_get_flush_tile": ([vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pqmc_batch_set_scan_chunk": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_get_scan_chunk": ([vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pqmc_batch_set_gemm_engine": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_get_gemm_engine": ([vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "pqmc_batch_sweep_slices": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "pqmc_sweep_slices": ([vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "pqmc_set_field_slices": ([vp, ctypes.c_int, ctypes.c_int, _f64p], ctypes.c_int),
        "pqmc_get_field_slices": ([vp, ctypes.c_int, ctypes.c_int, _f64p], ctypes.c_int),
        "pqmc_batch_init": ([vp], ctypes.c_int),
        "pqmc_batch_stream": ([vp, ctypes.POINTER(vp)], ctypes.c_int),
        "pqmc_batch_info": ([vp, _i32p], ctypes.c_int),
        "pqmc_batch_set_timing": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_get_timing": ([vp, _f64p, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "pqmc_batch_flush_rounds": ([vp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "pqmc_batch_scan_profile": ([vp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "pqmc_batch_set_graphs": ([vp, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_classes": ([vp, _i32p], ctypes.c_int),
        "pqmc_batch_field_slices": ([vp, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int], ctypes.c_int),
        "pqmc_batch_states": ([vp, ctypes.POINTER(PqmcState)], ctypes.c_int),
        "pqmc_batch_class_info": ([vp, ctypes.c_int, _i32p], ctypes.c_int),
        "pqmc_batch_graph_count": ([vp, _i32p], ctypes.c_int),
        "pqmc_exact_update_check": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _f64p, _f64p], ctypes.c_int),
        "pqmc_exact_update_check_tile": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, _i32p, _f64p, _f64p, ctypes.c_int],
                                         ctypes.c_int),
        "pqmc_recompute_gemm_check": ([ctypes.c_char, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, _f64p, ctypes.c_int, _f64p, ctypes.c_int, _f64p, ctypes.c_int,
                                       ctypes.c_int], ctypes.c_int),
        "pqmc_version": ([], ctypes.c_char_p),
        "pqmc_last_error": ([], ctypes.c_char_p),
        "pqmc_kernel_launches": ([], ctypes.c_int64),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes, fn.restype = args, res
    if path is None:
        _LIB = lib
    return lib


def exported_symbols_from_header(header: str) -> list[str]:
    """Names of every function declared in include/pqmc_gb300.h."""
    import re
    txt = open(header).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|int64_t)\s+(pqmc_\w+)\s*\(", txt, re.M)))


class PqmcError(RuntimeError):
    pass


def check(lib, status: int, what: str):
    if status != PQMC_OK:
        msg = lib.pqmc_last_error()
        raise PqmcError(f"{what} failed: {ERRORS.get(status, status)}: "
                        f"{msg.decode() if msg else ''}")
