"""Host-side model set-up: the reference's initialisation, restated in Python.

This module builds, on the host, every table the hot path reads:

* a reader for the reference's Fortran namelist model files
  (``general_paramter_init``, src/input.f90:218-262, and the model groups of
  input/model/*.nml);
* the lattice (src/mod_lattice.f90:6-205);
* the plaquette tables of every phonon-field family
  (``set_typed_pf``, src/mod_phonon_field.f90:249-421);
* the derived parameters of ``init`` (src/input.f90:167-205) and
  ``init_pf_para`` (:207-216);
* the trial Slater state (``set_k_slater`` / ``set_nelec_occupied``,
  src/Main_PQMC.f90:248-305);
* the initial boson field (``init_boson_field``, src/Main_PQMC.f90:307-371),
  either the reference's own ran2-driven form or a seeded Gaussian.

None of this is on the hot path; it runs once per chain, like the
reference's set-up.  The result is a :class:`Model` whose arrays are handed
to the CUDA library through the ``pqmc_model`` C struct.
"""
from __future__ import annotations

import dataclasses
import math
import re
from typing import Any

import numpy as np

from .rng import Ran2

EXPKV_GENERAL, EXPKV_EPSOCZ, EXPKV_EPSOC, EXPKV_EPSOCZ_BLOCK = 0, 1, 2, 3
PROPOSAL_UNIFORM, PROPOSAL_GAUSSIAN = 0, 1
PI_SP = float(np.float32(math.pi))  # PI of src/mod_nrtype.f90:42 is REAL(SP)

# --------------------------------------------------------------------------
# Fortran namelist reader (the subset the reference's model files use)
# --------------------------------------------------------------------------
_TOKEN = re.compile(
    r"""\s*(?:
        (?P<cplx>\(\s*[^(),]+\s*,\s*[^(),]+\s*\)) |
        (?P<str>"[^"]*"|'[^']*') |
        (?P<word>[^\s,/=()]+)
    )\s*,?""",
    re.X,
)


def _strip_comments(text: str) -> str:
    out = []
    for line in text.splitlines():
        buf, q = [], None
        for ch in line:
            if q:
                buf.append(ch)
                if ch == q:
                    q = None
            elif ch in "\"'":
                q = ch
                buf.append(ch)
            elif ch == "!":
                break
            else:
                buf.append(ch)
        out.append("".join(buf))
    return "\n".join(out)


def _scalar(tok: str) -> Any:
    t = tok.strip()
    lo = t.lower()
    if lo in (".true.", "t", ".t.", "true"):
        return True
    if lo in (".false.", "f", ".f.", "false"):
        return False
    if t.startswith(("'", '"')):
        return t[1:-1]
    if t.startswith("("):
        re_, im_ = t[1:-1].split(",")
        return complex(_scalar(re_), _scalar(im_))
    try:
        return int(t)
    except ValueError:
        return float(lo.replace("d", "e"))


def parse_namelists(text: str) -> list[tuple[str, dict[str, Any]]]:
    """All namelist groups of a file, in file order: [(name, {key: value})].

    A value is a scalar when one item is given, else a list.  Keys are lower
    case.  Group order matters: the reference reads repeated groups
    (``pf_pos``/``pf_K``/``pf_V``) sequentially from the file position
    (src/mod_phonon_field.f90:138-191)."""
    text = _strip_comments(text)
    groups = []
    for m in re.finditer(r"&(\w+)(.*?)(?<![\w.])/", text, re.S):
        name, body = m.group(1).lower(), m.group(2)
        parts = re.split(r"(\b[A-Za-z_]\w*\s*=)", body)
        d: dict[str, Any] = {}
        for i in range(1, len(parts), 2):
            key = parts[i].rstrip("= \t\n").lower()
            vals = [
                _scalar(mm.group(mm.lastgroup))
                for mm in _TOKEN.finditer(parts[i + 1])
                if mm.lastgroup
            ]
            d[key] = vals[0] if len(vals) == 1 else vals
        groups.append((name, d))
    return groups


class _Reader:
    """Sequential namelist reads (Fortran READ(unit, nml=...))."""

    def __init__(self, groups):
        self.groups, self.pos = groups, 0

    def rewind(self):
        self.pos = 0

    def read(self, name: str, required: bool = True) -> dict[str, Any]:
        for i in range(self.pos, len(self.groups)):
            if self.groups[i][0] == name.lower():
                self.pos = i + 1
                return self.groups[i][1]
        if required:
            raise ValueError(f"namelist group &{name} not found")
        return {}


def _as_list(v) -> list:
    return list(v) if isinstance(v, (list, tuple)) else [v]


# --------------------------------------------------------------------------
# model description
# --------------------------------------------------------------------------
@dataclasses.dataclass
class PfSpec:
    """One phonon-field family (one &pf_pos/&pf_K/&pf_V triple)."""

    dim: int
    n_cover: float
    tsl: list[int]            # pla_tsl_dvec_uc, flat, column-major (d,d)
    offset: list[int]         # pla_offset_dvec_uc (d)
    int_subsites: list[int]   # pla_int_subsites, flat, column-major (d+1,dim)
    k_exist: bool = True
    v_exist: bool = True
    k_coe: complex = 1.0
    kmat: list[complex] | None = None   # flat column-major (dim,dim)
    v_coe: complex = 0.0
    vmat: list[complex] | None = None
    bf_index: int = 1


@dataclasses.dataclass
class ModelSpec:
    """Everything the reference reads from a model namelist."""

    lat_dim: int
    n_subsite: int
    lat_size: list[int]
    lat_vec: list[float]
    site_vec: list[float]
    periodic: list[bool]
    bc_phase: list[float]               # in units of pi
    pfs: list[PfSpec]
    slater: PfSpec
    bf_sets: int
    model_name: str = "EPSOCZ"
    delt: float = 0.1
    beta: float = 8.0
    ngroup: int = 5
    filling: float = 0.5
    ncopy: int = 1
    hop: float = 1.0
    D: float = 1.0
    M: float = 1.0
    omega: float = 1.0
    ep_parameter: float = 1.0
    jump_distance: float = 1.0
    n_local_update: int = 1
    metropolis: bool = True
    greatest_decent: bool = False
    local_update: bool = True
    tr_weight: bool = False
    tr_slater: bool = True
    biased_phonon: float = 0.0
    random_range: float = 0.25
    offset: float = 0.05
    phase_intra_cell: list[complex] = dataclasses.field(default_factory=lambda: [1, -1])
    phase_k_inter_cell: list[float] = dataclasses.field(default_factory=lambda: [1, 1])
    observables: list[tuple[str, str]] = dataclasses.field(default_factory=list)
    warmup: int = 0
    meas_interval: int = 1
    meas_number: int = 0
    nbin_per_core: int = 1
    nmeas_per_bin: int = 1
    expkv_kind: int | None = None       # None: chosen from model_name
    proposal_kind: int = PROPOSAL_UNIFORM


def spec_from_namelist(text: str, model_name: str = "EPSOCZ") -> ModelSpec:
    """Read a reference model namelist file (input/model/*.nml layout)."""
    groups = parse_namelists(text)
    rd = _Reader(groups)
    ga = rd.read("general_arguments"); rd.rewind()
    cv = rd.read("control_varibles"); rd.rewind()
    mc = rd.read("mc_parameter"); rd.rewind()
    ph = rd.read("phonon_arguments"); rd.rewind()
    ld = rd.read("lat_dim")
    ls = rd.read("lat_spatial")
    lsv = rd.read("lat_subsite_vector")
    lbc = rd.read("lat_boundary_condition")
    rd.rewind()
    sl = rd.read("slater")
    sld = rd.read("slater_detail")
    rd.rewind()
    pb = rd.read("pf_basic")
    n_pf = int(ph["n_phonon_field"])
    ids = _as_list(pb.get("id", list(range(1, n_pf + 1))))
    kex = _as_list(pb.get("k_exist", [False] * n_pf))
    vex = _as_list(pb.get("v_exist", [False] * n_pf))
    dims = _as_list(pb["pf_dim"])
    cov = _as_list(pb["n_cover"])
    rd.rewind()
    pfs = []
    for i in range(n_pf):
        pos = rd.read("pf_pos")
        pk = rd.read("pf_k") if kex[i] else {}
        pv = rd.read("pf_v") if vex[i] else {}
        dim = int(dims[i])
        pfs.append(
            PfSpec(
                dim=dim,
                n_cover=float(cov[i]),
                tsl=[int(v) for v in _as_list(pos["pla_tsl_dvec_uc"])],
                offset=[int(v) for v in _as_list(pos["pla_offset_dvec_uc"])],
                int_subsites=[int(v) for v in _as_list(pos["pla_int_subsites"])],
                k_exist=bool(kex[i]),
                v_exist=bool(vex[i]),
                k_coe=complex(pk.get("k_coe", 0.0)),
                kmat=[complex(v) for v in _as_list(pk.get("kmatrix", [0.0] * dim * dim))],
                v_coe=complex(pv.get("v_coe", 0.0)),
                vmat=[complex(v) for v in _as_list(pv.get("vmatrix", [0.0] * dim * dim))],
                bf_index=int(pv.get("bf_index", 0)),
            )
        )
        assert ids[i] == i + 1, "family ids must be 1..n_phonon_field in order"
    rd.rewind()
    bb = rd.read("bf_basics")
    bi = rd.read("bf_initial", required=False)
    obs = [(d["name"], d["obskind"]) for n, d in groups if n == "observable"]
    sdim = int(sl["pf_dim"])
    slater = PfSpec(
        dim=sdim,
        n_cover=float(sl["n_cover"]),
        tsl=[int(v) for v in _as_list(sld["pla_tsl_dvec_uc"])],
        offset=[int(v) for v in _as_list(sld["pla_offset_dvec_uc"])],
        int_subsites=[int(v) for v in _as_list(sld["pla_int_subsites"])],
        k_exist=True,
        v_exist=False,
        k_coe=complex(sld.get("k_coe", 0.0)),
        kmat=[complex(v) for v in _as_list(sld["kmatrix"])],
    )
    d = int(ld["dim"])
    return ModelSpec(
        lat_dim=d,
        n_subsite=int(ld["n_subsite_uc"]),
        lat_size=[int(v) for v in _as_list(ls["lat_size"])],
        lat_vec=[float(v) for v in _as_list(ls["lat_vec"])],
        site_vec=[float(v) for v in _as_list(lsv["site_vec"])],
        periodic=[bool(v) for v in _as_list(lbc["periodic"])],
        bc_phase=[float(v) for v in _as_list(lbc["bc_phase"])],
        pfs=pfs,
        slater=slater,
        bf_sets=int(bb["bf_sets"]),
        model_name=model_name,
        delt=float(ga.get("delt", 0.1)),
        beta=float(ga.get("beta", 90.0)),
        ngroup=int(ga.get("ngroup", 5)),
        filling=float(ga.get("filling", 1.0)),
        ncopy=int(ga.get("ncopy", 1)),
        D=float(ph.get("d", 1.0)),
        M=float(ph.get("m", 1.0)),
        omega=float(ph.get("omega", 1.0)),
        ep_parameter=float(ph.get("ep_parameter", 1.0)),
        jump_distance=float(ph.get("jump_distance", 1.0)),
        n_local_update=int(ph.get("n_local_update", 1)),
        metropolis=bool(cv.get("metropolis", True)),
        greatest_decent=bool(cv.get("greatest_decent", False)),
        local_update=bool(cv.get("local_update", True)),
        tr_weight=bool(cv.get("tr_weight", False)),
        tr_slater=bool(cv.get("tr_slater", True)),
        random_range=float(bi.get("random_range", 0.0)),
        offset=float(bi.get("offset", 0.0)),
        phase_intra_cell=[complex(v) for v in _as_list(bi.get("phase_intra_cell", [1] * int(bb["bf_sets"])))],
        phase_k_inter_cell=[float(v) for v in _as_list(bi.get("phase_k_inter_cell", [0] * d))],
        observables=obs,
        warmup=int(mc.get("warmup", 0)),
        meas_interval=int(mc.get("meas_interval", 1)),
        meas_number=int(mc.get("meas_number", 0)),
        nbin_per_core=int(mc.get("nbin_per_core", 1)),
        nmeas_per_bin=int(mc.get("nmeas_per_bin", 1)),
    )


# --------------------------------------------------------------------------
# EPSOCZ-type model written out directly (the structure of
# input/model/EPSOCZ.nml: two spin sub-sites per cell, four checkerboard
# families of 4-site bond plaquettes, x bonds coupled to -i sigma_y, y bonds
# to -i sigma_x).  `alpha` adds a static spin-orbit term of the same matrix
# form to the hopping block, which keeps h^H h proportional to 1.
# --------------------------------------------------------------------------
_MY = [0, 0, 0, -1, 0, 0, 1, 0, 0, 1, 0, 0, -1, 0, 0, 0]          # -i sigma_y block
_MX = [0, 0, 0, -1j, 0, 0, -1j, 0, 0, 1j, 0, 0, 1j, 0, 0, 0]      # -i sigma_x block
_KB = [0, 0, 1, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 1, 0, 0]            # spin-diagonal hop


def epsocz_spec(L: int | tuple[int, int] = 4, *, lam: float = 1.0, alpha: float = 0.0,
                omega: float = 1.0, delt: float = 0.1, ntime: int = 80, ngroup: int = 10,
                filling: float = 0.5, jump_distance: float = 0.5, bc_phase=(0.0, 0.0),
                hop: float = 1.0, proposal_kind: int = PROPOSAL_UNIFORM) -> ModelSpec:
    La, Lb = (L, L) if isinstance(L, int) else L
    pfs = []
    for vert, off in ((False, (0, 0)), (False, (1, 0)), (True, (0, 0)), (True, (0, 1))):
        v = _MX if vert else _MY
        # K block I + s*alpha*V with s chosen so that K_coe*K = -I + alpha*V,
        # K_coe = -hop: K = I - (alpha/hop)*V on the off-diagonal blocks.
        k = [complex(kb) - (alpha / hop) * complex(vv) for kb, vv in zip(_KB, v)]
        pfs.append(PfSpec(
            dim=4, n_cover=1.0, tsl=[2, 0, 1, 1], offset=list(off),
            int_subsites=([0, 0, 1, 0, 0, 2, 0, 1, 1, 0, 1, 2] if vert
                          else [0, 0, 1, 0, 0, 2, 1, 0, 1, 1, 0, 2]),
            k_exist=True, v_exist=True, k_coe=1.0, kmat=k, v_coe=1.0,
            vmat=[complex(x) for x in v], bf_index=2 if vert else 1))
    sk = [0j] * 36
    for (i, j, val) in ((1, 1, 10), (3, 1, 1), (5, 1, 1), (4, 2, 1), (6, 2, 1), (1, 3, 1),
                        (3, 3, 10), (2, 4, 1), (1, 5, 1), (5, 5, 10), (2, 6, 1)):
        sk[(i - 1) + 6 * (j - 1)] = complex(val)
    slater = PfSpec(dim=6, n_cover=3.0, tsl=[1, 0, 0, 1], offset=[0, 0],
                    int_subsites=[0, 0, 1, 0, 0, 2, 1, 0, 1, 1, 0, 2, 0, 1, 1, 0, 1, 2],
                    k_exist=True, v_exist=False, k_coe=1.0, kmat=sk)
    kind = EXPKV_EPSOCZ if alpha == 0.0 else EXPKV_EPSOCZ_BLOCK
    return ModelSpec(
        lat_dim=2, n_subsite=2, lat_size=[La, Lb], lat_vec=[1, 0, 0, 1], site_vec=[0, 0, 0, 0],
        periodic=[True, True], bc_phase=list(bc_phase), pfs=pfs, slater=slater, bf_sets=2,
        model_name="EPSOCZ", delt=delt, beta=ntime * delt, ngroup=ngroup, filling=filling,
        hop=hop, D=1.0, M=1.0, omega=omega, ep_parameter=lam, jump_distance=jump_distance,
        tr_slater=True, expkv_kind=kind, proposal_kind=proposal_kind,
        observables=[(n, "scalar") for n in ("BF_KE", "BF_PE", "BF_X")] +
                    [(n, "field") for n in FIELD_NAMES])


FIELD_NAMES = [
    "BFx_BFx", "BFx_BFy", "BFy_BFy", "BFxy_BFxy", "Jxx_Jxx", "Jxy_Jxy", "Jyx_Jyx", "Jyy_Jyy",
    "Jxx_Jyx", "Jxy_Jyy", "Jxxh_Jxxh", "Jxyh_Jxyh", "Jyxh_Jyxh", "Jyyh_Jyyh", "Jxxh_Jyxh",
    "Jxyh_Jyyh", "Jxxh_Jyyh", "Jxyh_Jyxh", "den_den", "SC_SC", "Sz_Sz", "Sx_Sx", "Sy_Sy",
    "cJyx_cJyx", "cJxy_cJxy",
]
SCALAR_NAMES = ["BF_KE", "BF_PE", "BF_X"]


# --------------------------------------------------------------------------
# built model
# --------------------------------------------------------------------------
@dataclasses.dataclass
class Lattice:
    dim: int
    n_sub: int
    dlength: np.ndarray
    tsl_rvec: np.ndarray          # (dim,dim), columns are lattice vectors
    n_cell: int
    ns: int
    bc_phase: np.ndarray          # complex (dim)
    cell_dpos: np.ndarray         # (n_cell,dim) 0-based
    cell_rpos: np.ndarray         # (n_cell,dim)
    k_phase: np.ndarray           # complex (n_cell,n_cell)

    def cell_sites(self, c: int) -> list[int]:
        """0-based sites of 0-based cell c (sites(j) = (i-1)*n_sub + j)."""
        return [c * self.n_sub + j for j in range(self.n_sub)]

    def uc_index(self, dpos) -> int:
        """get_uc_index_from_dpos (src/mod_lattice.f90:256-280), 0-based."""
        ind, mul = 0, 1
        for i in range(self.dim):
            v = int(dpos[i])
            if v < -0.00001:
                v += int(self.dlength[i])
            v = v % int(self.dlength[i])
            ind += v * mul
            mul *= int(self.dlength[i])
        return ind


def build_lattice(spec: ModelSpec) -> Lattice:
    """readin_lattice_para + setup_lattice + calculate_1stBZ
    (src/mod_lattice.f90:15-205)."""
    d = spec.lat_dim
    dl = np.array(spec.lat_size[:d], dtype=np.int64)
    tsl = np.array(spec.lat_vec[: d * d], dtype=np.float64).reshape((d, d), order="F")
    n_cell = int(np.prod(dl))
    bc = np.array([np.exp(1j * spec.bc_phase[i] * math.acos(-1.0)) if spec.periodic[i] else 0.0
                   for i in range(d)], dtype=np.complex128)
    dpos = np.zeros((n_cell, d), dtype=np.int64)
    for i in range(n_cell):
        t = i
        for k in range(d):
            dpos[i, k] = t % dl[k]
            t = (t - dpos[i, k]) // dl[k]
    rpos = dpos @ tsl.T
    kvec = np.linalg.inv(tsl.T) * 2.0 * math.acos(-1.0)
    if kvec[:, 0] @ tsl[:, 0] / (np.linalg.norm(kvec[:, 0]) * np.linalg.norm(tsl[:, 0])) < -1e-5:
        kvec[:, 0] = -kvec[:, 0]
    for i in range(d):
        if kvec[:, i] @ kvec[:, 0] / (np.linalg.norm(kvec[:, i]) * np.linalg.norm(kvec[:, 0])) < -1e-5:
            kvec[:, i] = -kvec[:, i]
    k_off = np.zeros(d)
    dk = np.zeros((d, d))
    for i in range(d):
        k_off = k_off + (dl[i] % 2) * kvec[:, i] / dl[i] / 2.0
        k_off = k_off - 0.5 * kvec[:, i]
        dk[:, i] = kvec[:, i] / dl[i]
    fbz = dpos @ dk.T + k_off           # FBZ(:,ik) for k index laid out like cells
    k_phase = np.exp(1j * (fbz @ rpos.T))
    return Lattice(d, spec.n_subsite, dl, tsl, n_cell, n_cell * spec.n_subsite, bc, dpos, rpos, k_phase)


@dataclasses.dataclass
class PfTables:
    dim: int
    n_pla: int
    site_list: np.ndarray      # (n_pla, dim) 0-based
    crossing: np.ndarray       # (n_pla,) bool
    bc_phases: np.ndarray      # (n_pla, dim, dim) complex
    bf_list: np.ndarray        # (n_pla,) 0-based


def set_typed_pf(lat: Lattice, pf: PfSpec, bf_sets: int) -> PfTables:
    """Plaquette site lists, boundary phases and boson indices of one family
    (set_typed_pf, src/mod_phonon_field.f90:249-421)."""
    d, dim = lat.dim, pf.dim
    n_pla = int(lat.ns * pf.n_cover / dim)
    tsl = np.array(pf.tsl[: d * d], dtype=np.float64).reshape((d, d), order="F")
    inv = np.linalg.inv(tsl)
    off = np.array(pf.offset[:d], dtype=np.int64)
    isub = np.array(pf.int_subsites[: (d + 1) * dim], dtype=np.int64).reshape((d + 1, dim), order="F")
    sites = -np.ones((n_pla, dim), dtype=np.int64)
    cnt = 0
    for c in range(lat.n_cell):
        cd = lat.cell_dpos[c] - off
        for j in range(d):
            if cd[j] < -0.0001:
                cd[j] += lat.dlength[j]
            if cd[j] >= lat.dlength[j] - 0.0001:
                cd[j] -= lat.dlength[j]
        xp = inv @ cd
        if np.any(np.abs(np.rint(xp) - xp) > 1e-6):
            continue
        if cnt >= n_pla:
            raise ValueError("set_typed_pf: plaquette count exceeds n_plaquette")
        sites[cnt, 0] = lat.cell_sites(c)[isub[d, 0] - 1]
        cnt += 1
    crossing = np.zeros(n_pla, dtype=bool)
    bcp = np.ones((n_pla, dim, dim), dtype=np.complex128)
    if dim > 1:
        for p in range(n_pla):
            pos = lat.cell_dpos[sites[p, 0] // lat.n_sub]
            for i in range(1, dim):
                cd = pos + isub[:d, i]
                for j in range(d):
                    if cd[j] > lat.dlength[j] - 0.0001:
                        cd[j] -= lat.dlength[j]
                    if cd[j] < -0.0001:
                        cd[j] += lat.dlength[j]
                sites[p, i] = lat.cell_sites(lat.uc_index(cd))[isub[d, i] - 1]
        for p in range(n_pla):
            for i in range(dim):
                for j in range(dim):
                    idp = lat.cell_dpos[sites[p, i] // lat.n_sub]
                    jd = idp - isub[:d, i] + isub[:d, j]
                    for k in range(d):
                        if jd[k] >= lat.dlength[k] - 0.0001:
                            crossing[p] = True
                            bcp[p, i, j] *= lat.bc_phase[k]
                        if jd[k] < -0.0001:
                            crossing[p] = True
                            bcp[p, i, j] *= np.conj(lat.bc_phase[k])
    bfl = np.array([(pf.bf_index - 1) + (sites[p, 0] // lat.n_sub) * bf_sets for p in range(n_pla)],
                   dtype=np.int64)
    return PfTables(dim, n_pla, sites, crossing, bcp, bfl)


@dataclasses.dataclass
class Model:
    spec: ModelSpec
    lat: Lattice
    pf: list[PfTables]
    ntime: int
    ngroup: int
    nblock: int
    ns: int
    nelec: int
    n_bf: int
    M: float
    D: float
    char_length: float
    jump_distance: float
    k_coe: np.ndarray            # complex (n_pf) after init_pf_para
    v_coe: np.ndarray
    kmat: np.ndarray             # complex (n_pf, pdim, pdim)
    vmat: np.ndarray
    pdim: int
    max_pla: int
    expkv_kind: int
    slater_q: np.ndarray | None = None   # (Ns, nelec) complex, Fortran order
    slater_d: np.ndarray | None = None   # (nelec,) complex

    # flat arrays in the pqmc_model layout -------------------------------
    def flat_tables(self) -> dict[str, np.ndarray]:
        npf, pd, mp = len(self.pf), self.pdim, self.max_pla
        site = np.zeros((npf, mp, pd), dtype=np.int32)
        bfl = np.zeros((npf, mp), dtype=np.int32)
        cross = np.zeros((npf, mp), dtype=np.int32)
        bcp = np.ones((npf, mp, pd, pd), dtype=np.complex128)
        for f, t in enumerate(self.pf):
            site[f, : t.n_pla, : t.dim] = t.site_list
            bfl[f, : t.n_pla] = t.bf_list
            cross[f, : t.n_pla] = t.crossing
            # Fortran (i,j,pla,pf) column-major == C [pf][pla][j][i]
            bcp[f, : t.n_pla, : t.dim, : t.dim] = np.transpose(t.bc_phases, (0, 2, 1))
        return dict(
            pla_site_list=np.ascontiguousarray(site),
            bf_list=np.ascontiguousarray(bfl),
            boundary_crossing=np.ascontiguousarray(cross),
            bc_phases=np.ascontiguousarray(bcp),
            kmat=np.ascontiguousarray(np.transpose(self.kmat, (0, 2, 1))),
            vmat=np.ascontiguousarray(np.transpose(self.vmat, (0, 2, 1))),
        )


def build_model(spec: ModelSpec, *, with_slater: bool = True, twist_seed: int | None = None,
                twist: float = 0.0) -> Model:
    """Lattice + families + derived parameters (+ trial state)."""
    lat = build_lattice(spec)
    tables = [set_typed_pf(lat, p, spec.bf_sets) for p in spec.pfs]
    ntime = int(round(spec.beta / spec.delt))
    # init (src/input.f90:167-205)
    D = 1.0
    M = D * spec.omega ** (-2)
    if M < 0.001:
        M = 0.0
        char_length = math.sqrt(1.0 / (D * spec.ep_parameter))
    else:
        char_length = 1.0 / (M * spec.omega)
    jump = spec.jump_distance * (0.1 / spec.delt) * char_length
    nelec = int(round(lat.ns * spec.filling))
    pdim = max(p.dim for p in spec.pfs)
    max_pla = max(t.n_pla for t in tables)
    npf = len(spec.pfs)
    kmat = np.zeros((npf, pdim, pdim), dtype=np.complex128)
    vmat = np.zeros((npf, pdim, pdim), dtype=np.complex128)
    for f, p in enumerate(spec.pfs):
        kmat[f, : p.dim, : p.dim] = np.array(p.kmat, dtype=np.complex128).reshape((p.dim, p.dim), order="F")
        vmat[f, : p.dim, : p.dim] = np.array(p.vmat, dtype=np.complex128).reshape((p.dim, p.dim), order="F")
    # init_pf_para (src/input.f90:207-216)
    k_coe = np.array([complex(p.k_coe) * (-spec.hop) for p in spec.pfs], dtype=np.complex128)
    v_coe = np.array([complex(p.v_coe) * spec.ep_parameter for p in spec.pfs], dtype=np.complex128)
    kind = spec.expkv_kind
    if kind is None:
        kind = {"EPSOCZ": EXPKV_EPSOCZ, "EPSOC": EXPKV_EPSOC}.get(spec.model_name.strip(), EXPKV_GENERAL)
    m = Model(spec, lat, tables, ntime, spec.ngroup, ntime // spec.ngroup + 2, lat.ns, nelec,
              spec.bf_sets * lat.n_cell, M, D, char_length, jump, k_coe, v_coe, kmat, vmat, pdim,
              max_pla, kind)
    if with_slater:
        m.slater_q, m.slater_d = slater_state(m, twist_seed=twist_seed, twist=twist)
    return m


def k_slater(m: Model, twist_seed: int | None = None, twist: float = 0.0) -> np.ndarray:
    """set_k_slater (src/Main_PQMC.f90:248-277): K_slater(S,S) = K_coe*Kmatrix
    (times BC phases), later plaquettes overwrite earlier ones.  An optional
    seeded random twist of relative size `twist` on every bond lifts shell
    degeneracies of the trial state deterministically."""
    spec = m.spec
    t = set_typed_pf(m.lat, spec.slater, spec.bf_sets)
    kc = complex(spec.slater.k_coe) * (-spec.hop)
    km = np.array(spec.slater.kmat, dtype=np.complex128).reshape((t.dim, t.dim), order="F")
    K = np.zeros((m.ns, m.ns), dtype=np.complex128)
    for p in range(t.n_pla):
        blk = kc * km
        if t.crossing[p]:
            blk = blk * t.bc_phases[p]
        S = t.site_list[p]
        K[np.ix_(S, S)] = blk
    if twist and twist_seed is not None:
        rng = np.random.default_rng(twist_seed)
        noise = rng.uniform(-1.0, 1.0, size=K.shape)
        noise = 0.5 * (noise + noise.T)
        K = K + twist * np.where(K != 0, noise * np.abs(K), 0.0)
        K = 0.5 * (K + K.conj().T)
    return K


def slater_state(m: Model, twist_seed: int | None = None, twist: float = 0.0):
    """set_nelec_occupied (src/Main_PQMC.f90:279-305): lowest eigenvectors of
    K_slater (time-reversal partners for the second half when TR_slater),
    then QDR (zqdr, src/mod_matrixlib.f90:323-334)."""
    K = k_slater(m, twist_seed, twist)
    w, v = np.linalg.eigh(K)
    ne = m.nelec
    if m.spec.tr_slater:
        half = ne // 2
        tr = np.zeros((m.ns, m.ns))
        for i in range(0, m.ns - 1, 2):
            tr[i, i + 1] = 1.0
            tr[i + 1, i] = -1.0
        sl = np.concatenate([v[:, :half], np.conj(tr @ v[:, :half])], axis=1)
    else:
        sl = v[:, :ne]
    q, r = np.linalg.qr(sl)
    d = np.diag(r).copy()
    return np.asfortranarray(q), d


# --------------------------------------------------------------------------
# boson field initialisation
# --------------------------------------------------------------------------
def field_reference_init(m: Model, rng: Ran2) -> np.ndarray:
    """init_boson_field without import (src/Main_PQMC.f90:329-349): uniform
    random_range*ran_sysm() + phase*offset, consuming ran2 draws in
    (time, cell, boson) order.  Returns boson_field(n_bf, ntime) in Fortran
    order."""
    spec, lat = m.spec, m.lat
    rr = 0.5 * spec.random_range * m.char_length
    off = 0.5 * spec.offset * m.char_length
    f = np.zeros((m.n_bf, m.ntime), dtype=np.float64, order="F")
    pk = np.array(spec.phase_k_inter_cell[: lat.dim], dtype=np.float64)
    phases = [np.exp(1j * float(np.sum(pk * lat.cell_rpos[c] * PI_SP))) for c in range(lat.n_cell)]
    for t in range(m.ntime):
        for c in range(lat.n_cell):
            for b in range(spec.bf_sets):
                r = float(rng.ran_sysm())
                val = (rr * r + phases[c] * off) * complex(spec.phase_intra_cell[b])
                f[b + c * spec.bf_sets, t] = val.real
    return f


def field_gaussian(m: Model, seed: int, sigma: float = 0.5) -> np.ndarray:
    """x_{b,tau} i.i.d. N(0, sigma^2) from numpy's PCG64 seeded with `seed`
    (the seeded synthetic initial fields of the benchmark configurations)."""
    g = np.random.default_rng(seed)
    return np.asfortranarray(g.normal(0.0, sigma, size=(m.n_bf, m.ntime)))


# --------------------------------------------------------------------------
# measurement layout (ms_take_measurement, src/mod_meas.f90:237-289)
# --------------------------------------------------------------------------
def meas_tables(m: Model) -> dict[str, np.ndarray]:
    lat = m.lat
    if lat.dim != 2 or lat.n_sub != 2 or m.spec.bf_sets != 2:
        raise ValueError("equal-time measurement needs 2 sub-sites and 2 bosons per cell in 2D")
    nc = lat.n_cell
    sites = np.array([lat.cell_sites(c) for c in range(nc)], dtype=np.int32)        # (nc,2)
    bf = np.array([[2 * c, 2 * c + 1] for c in range(nc)], dtype=np.int32)
    xnb = np.array([lat.uc_index(lat.cell_dpos[c] + np.array([1, 0])) for c in range(nc)], dtype=np.int32)
    ynb = np.array([lat.uc_index(lat.cell_dpos[c] + np.array([0, 1])) for c in range(nc)], dtype=np.int32)
    cross = np.array([[int(lat.cell_dpos[c, i] == lat.dlength[i] - 1) for i in range(2)] for c in range(nc)],
                     dtype=np.int32)
    rel = np.zeros((nc, nc), dtype=np.int32)    # [c2][c1] -> Fortran rel(c1,c2)
    for c1 in range(nc):
        for c2 in range(nc):
            dr = [(lat.cell_dpos[c2, i] - lat.cell_dpos[c1, i] + lat.dlength[i]) % lat.dlength[i]
                  for i in range(2)]
            rel[c2, c1] = lat.uc_index(dr)
    return dict(cell_sites=sites, cell_bf=bf, cell_xnb=xnb, cell_ynb=ynb, cell_cross=cross,
                rel_index=rel, bc_phase=lat.bc_phase.astype(np.complex128),
                k_phase=np.ascontiguousarray(lat.k_phase.T))   # C [ic][ik] == Fortran (ik,ic)


def record_width(m: Model) -> int:
    return len(SCALAR_NAMES) + 2 * len(FIELD_NAMES) * m.lat.n_cell
