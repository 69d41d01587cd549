"""Phonon-field files and checkpoint/resume of chains and batches.

Field files follow the reference's import_ph_field format
(src/Main_PQMC.f90:355-369): one record per time slice, time = 1..ntime,
each record the n_bf values boson_field(:, time) in Fortran ``f18.6``
(18 characters, 6 decimals, right-aligned).  The file is named
``ph_field_.dat`` (``ph_field_core1.dat`` in MPI builds, which all read
core 1's file).  The reference reads these files but never writes them
(the writer call is commented out at :166); ``write_ph_field`` produces
the same layout, so a GPU run can seed a reference run and vice versa.
Six decimals lose precision: a checkpoint therefore stores the exact
doubles instead.

A checkpoint (``save_checkpoint``) holds, per chain, the exact boson field,
the ran2 state, the accept counters and the error maxima, plus the sweep
index `loop` it was taken after.  Resuming rebuilds expKV and G from the
field (init_expKV, init_g_T0(1)), which is what a fresh start of the
reference does, so it is valid at the start of a backward sweep: after an
even `loop` (a forward sweep ends where init_g_T0(1) starts).  The next
sweep to run is loop + 1.
"""
from __future__ import annotations

import numpy as np

FIELD_FILE = "ph_field_.dat"
FIELD_FILE_MPI = "ph_field_core1.dat"
_W = 18   # f18.6

FORMAT_VERSION = 1


def format_f18_6(x: float) -> str:
    """One value as Fortran F18.6 writes it (asterisks when it does not fit)."""
    s = f"{x:18.6f}"
    return "*" * _W if len(s) > _W else s


def write_ph_field(path: str, field: np.ndarray) -> None:
    """boson_field (n_bf, ntime) to a text file in the import_ph_field layout."""
    f = np.asarray(field, dtype=np.float64)
    if f.ndim != 2:
        raise ValueError("field must be (n_bf, ntime)")
    with open(path, "w") as out:
        for t in range(f.shape[1]):
            out.write("".join(format_f18_6(v) for v in f[:, t]) + "\n")


def read_ph_field(path: str, n_bf: int, ntime: int) -> np.ndarray:
    """The import_ph_field read (Main_PQMC.f90:365-367): ntime records of
    n_bf fixed-width F18.6 fields.  Returns (n_bf, ntime) float64."""
    out = np.zeros((n_bf, ntime), dtype=np.float64)
    with open(path) as f:
        for t in range(ntime):
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: {t} records, {ntime} expected")
            line = line.rstrip("\n")
            if len(line) < n_bf * _W:
                raise ValueError(f"{path}: record {t + 1} holds {len(line)} characters, {n_bf * _W} expected")
            for b in range(n_bf):
                fld = line[b * _W:(b + 1) * _W]
                if "*" in fld:
                    raise ValueError(f"{path}: record {t + 1}, field {b + 1} overflowed F18.6")
                out[b, t] = float(fld) if fld.strip() else 0.0
    return out


# ---------------------------------------------------------------------------
def _geometry(m) -> np.ndarray:
    return np.array([m.ns, m.nelec, m.ntime, m.ngroup, m.n_bf, len(m.pf)], dtype=np.int64)


def save_checkpoint(path: str, chains, loop: int) -> None:
    """Exact fields, ran2 states, counters and error maxima of `chains`
    (PqmcChain objects, e.g. ``PqmcBatch.chains``) after sweep `loop`."""
    if loop % 2 != 0:
        raise ValueError("checkpoints are taken after an even sweep (a completed forward sweep), "
                         "where init_g_T0(1) resumes")
    data = {"version": np.int64(FORMAT_VERSION), "loop": np.int64(loop), "n_chains": np.int64(len(chains))}
    for i, c in enumerate(chains):
        st = c.state()
        data[f"field_{i}"] = np.asarray(c.field(), dtype=np.float64)
        data[f"geometry_{i}"] = _geometry(c.m)
        data[f"rng_{i}"] = np.array(st["rng"], dtype=np.int32)
        data[f"counters_{i}"] = np.array([st["positive_accept"], st["negative_accept"]], dtype=np.int64)
        data[f"errors_{i}"] = np.array([st["err_fast_max"], st["err_fast"], st["err_g"], st["err_g_rel_max"]])
        data[f"ln_cw_{i}"] = np.array([st["ln_cw"].real, st["ln_cw"].imag])
    np.savez(path, **data)


def load_checkpoint(path: str) -> dict:
    """{loop, chains: [{field, geometry, state}]} of a saved checkpoint."""
    with np.load(path) as z:
        if int(z["version"]) != FORMAT_VERSION:
            raise ValueError(f"{path}: checkpoint format {int(z['version'])}, expected {FORMAT_VERSION}")
        out = {"loop": int(z["loop"]), "chains": []}
        for i in range(int(z["n_chains"])):
            pc, nc = (int(v) for v in z[f"counters_{i}"])
            e = z[f"errors_{i}"]
            lc = z[f"ln_cw_{i}"]
            out["chains"].append({
                "field": z[f"field_{i}"].copy(),
                "geometry": z[f"geometry_{i}"].copy(),
                "state": {"rng": [int(v) for v in z[f"rng_{i}"]], "positive_accept": pc, "negative_accept": nc,
                          "err_fast_max": float(e[0]), "err_fast": float(e[1]), "err_g": float(e[2]),
                          "err_g_rel_max": float(e[3]), "ln_cw": complex(lc[0], lc[1])},
            })
    return out


def _check_geometry(ck: dict, models) -> None:
    if len(ck["chains"]) != len(models):
        raise ValueError(f"checkpoint holds {len(ck['chains'])} chains, {len(models)} given")
    for i, (c, m) in enumerate(zip(ck["chains"], models)):
        if not np.array_equal(c["geometry"], _geometry(m)):
            raise ValueError(f"chain {i}: checkpoint geometry {c['geometry'].tolist()} does not match the model "
                             f"{_geometry(m).tolist()}")


def restore_chain(chain, ck: dict, i: int = 0) -> int:
    """Chain i of checkpoint `ck` into a PqmcChain of the same model; returns
    the next sweep to run."""
    _check_geometry({"chains": [ck["chains"][i]]}, [chain.m])
    c = ck["chains"][i]
    chain.set_field(c["field"])
    chain.set_state(c["state"])
    chain.init_expkv()
    chain.init_g(1)
    return ck["loop"] + 1


def restore_batch(batch, ck: dict) -> int:
    """Every chain of a PqmcBatch (same models, same order) from `ck`;
    returns the next sweep to run."""
    _check_geometry(ck, batch.models)
    for c, saved in zip(batch.chains, ck["chains"]):
        c.set_field(saved["field"])
        c.set_state(saved["state"])
    batch.init()
    return ck["loop"] + 1
