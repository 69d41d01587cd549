"""Measurement bins and output files in the reference's layout
(src/mod_meas.f90:587-627, 697-716, 729-763, 845-1017): offsets from the
observable namelist, bin means of the real part, tempout/out_core stream
files and the reading guide as the reference's post-processing parses it."""
import re

import numpy as np
import pytest

from pqmc_allinone_gb300 import model as M
from pqmc_allinone_gb300.output import KIND_FIELD, KIND_SCALAR, MeasurementBins, read_out_core, reference_layout
from tests.helpers import epsocz_small


def _parse_guide(path):
    """The namelist reading of the reference's post-processing: `key = value`
    lines of &basics and of every &obs group, values evaluated."""
    basics, obs, cur, group = {}, {}, None, None
    for line in open(path):
        s = line.strip()
        if s.startswith("&"):
            group, cur = s[1:], {}
            continue
        if s.startswith("/"):
            if group == "basics":
                basics = cur
            elif group == "obs":
                obs[cur["name"]] = cur
            group = None
            continue
        mt = re.match(r"(\w+)\s*=\s*(.*)", s)
        if mt and group:
            cur[mt.group(1)] = eval(mt.group(2))
    return basics, obs


def test_layout_of_the_full_namelist():
    m, _ = epsocz_small(L=4, ntime=20)
    lay = reference_layout(m)
    nc = m.lat.n_cell
    assert len(lay) == len(M.SCALAR_NAMES) + 2 * len(M.FIELD_NAMES)
    assert lay[0] == {"name": "BF_KE", "kind": KIND_SCALAR, "width": 1, "offset_lo": 1, "offset_hi": 1}
    assert lay[3]["name"] == "BFx_BFx" and lay[4]["name"] == "BFx_BFx_k" and lay[4]["kind"] == KIND_FIELD
    assert lay[-1]["offset_hi"] == M.record_width(m) == 3 + 2 * len(M.FIELD_NAMES) * nc
    for a, b in zip(lay, lay[1:]):
        assert b["offset_lo"] == a["offset_hi"] + 1


def test_bins_files_round_trip(tmp_path):
    m, _ = epsocz_small(L=4, ntime=20)
    w = M.record_width(m)
    rng = np.random.default_rng(3)
    recs = rng.normal(size=(6, w)) + 1j * rng.normal(size=(6, w))
    mb = MeasurementBins(m, nbins=3, nmeas=2, output_addr=str(tmp_path) + "/")
    mb.add_records(recs)
    with pytest.raises(RuntimeError):
        mb.add(recs[0])                                   # no more bins left
    mean = mb.finish()
    want = np.stack([mb.to_layout(recs[2 * b:2 * b + 2].mean(axis=0)).real for b in range(3)], axis=1)
    assert np.allclose(mean, want, rtol=0, atol=1e-15)
    basics, obs = _parse_guide(tmp_path / "data" / "reading_guide.nml")
    assert basics["n_obs"] == len(obs) == 53 and basics["total_width"] == w and basics["n_bins"] == 3
    assert basics["n_meas_per_bin"] == 2 and basics["field_width"] == m.lat.n_cell and basics["size_of_dp"] == 8
    assert obs["Sz_Sz_k"]["kind"] == 2 and obs["BF_X"]["offset_lo"] == 3
    back = read_out_core(str(tmp_path / "data" / "out_core.bin"), basics["total_width"], basics["n_bins"])
    assert np.array_equal(back, mean)
    tmp = np.fromfile(tmp_path / "temp" / "tempout_core.bin", dtype="<f8").reshape((w, 3), order="F")
    assert np.array_equal(tmp, mean)
    assert (tmp_path / "temp" / "tempout_core_count.dat").read_text().splitlines() == [
        "C   0   |    B   1", "C   0   |    B   2", "C   0   |    B   3"]
    mu, err = mb.estimate()
    assert np.allclose(mu, mean.mean(axis=1)) and np.all(err >= 0)


def test_subset_and_reordered_namelist(tmp_path):
    m, _ = epsocz_small(L=4, ntime=20)
    nc = m.lat.n_cell
    w = M.record_width(m)
    rec = np.arange(w, dtype=np.float64) + 0j
    obs = [("den_den", "field"), ("BF_X", "scalar"), ("no_such_obs", "scalar")]
    mb = MeasurementBins(m, nbins=1, nmeas=1, output_addr=str(tmp_path) + "/", core_id=5, observables=obs)
    assert mb.total_width == 2 * nc + 2
    mb.add(rec)
    mean = mb.finish()
    f = M.FIELD_NAMES.index("den_den")
    den, den_k = 3 + nc * f, 3 + nc * (len(M.FIELD_NAMES) + f)   # r-space block, then k-space block
    assert np.array_equal(mean[:nc, 0], rec[den:den + nc].real)
    assert np.array_equal(mean[nc:2 * nc, 0], rec[den_k:den_k + nc].real)
    assert mean[2 * nc, 0] == 2.0 and mean[2 * nc + 1, 0] == 0.0
    assert (tmp_path / "data" / "out_core5.bin").exists() and (tmp_path / "temp" / "tempout_core5.bin").exists()
    with pytest.raises(ValueError):
        reference_layout(m, [("a", "scalar"), ("a", "field")])


def test_oracle_record_in_the_namelist_layout(tmp_path):
    """A measurement record of the oracle (ms_begin_measure over a window of
    three slices) placed by name: every `<field>_k` slot holds the k-space
    transform (ms_k_space_obs, mod_meas.f90:546-566) of its `<field>` slot,
    and the scalars keep their values."""
    from oracle.oracle import OracleChain
    from tests.helpers import SEED_WORDS
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.8, alpha=0.3)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=True)
    o.init_expkv()
    o.init_g(1)
    half = m.ntime // 2
    rec = None
    for t in (half - 1, half, half + 1):
        rec = o.begin_measure(True, t, meas_number=1)
    assert rec is not None
    mb = MeasurementBins(m, nbins=1, nmeas=1, output_addr=str(tmp_path) + "/")
    v = mb.to_layout(rec)
    pos = {e["name"]: (e["offset_lo"] - 1, e["width"]) for e in mb.layout}
    nc = m.lat.n_cell
    for name in M.FIELD_NAMES:
        lo, w = pos[name]
        lk, wk = pos[name + "_k"]
        assert w == wk == nc
        r = v[lo:lo + w]
        want = (m.lat.k_phase @ r) / nc
        assert np.allclose(v[lk:lk + wk], want, rtol=1e-12, atol=1e-12 * (1 + np.abs(r).max())), name
    for i, name in enumerate(M.SCALAR_NAMES):
        assert v[pos[name][0]] == rec[i]
    assert np.abs(v).max() > 0


def _reference_readers(reference_root):
    """The reading functions of the reference's post-processing script
    (pprocess/check_core_data.py: read_namelist, read_obs_info,
    recalculate_k_data_function, transform_to_k_space), taken from its
    source by name; the script's module-level imports of plotting and
    parsing packages are not needed by these functions."""
    import ast
    import os
    import re as re_mod
    path = os.path.join(reference_root, "pprocess", "check_core_data.py")
    tree = ast.parse(open(path, encoding="utf-8").read())
    want = {"read_namelist", "read_obs_info", "recalculate_k_data_function", "transform_to_k_space"}
    mod = ast.Module(body=[n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in want],
                     type_ignores=[])
    ns = {"np": np, "os": os, "re": re_mod}
    exec(compile(mod, path, "exec"), ns)
    assert want <= set(ns)
    return ns


def test_files_read_by_the_reference_post_processing(tmp_path, reference_root):
    """Files written by MeasurementBins from oracle records, read back with
    the reference's own reader functions: the reading guide's basics and
    observable offsets, the out_core bin means, and the k-space slots as the
    reference's post-processing recomputes them from the r-space slots."""
    from oracle.oracle import OracleChain
    from tests.helpers import SEED_WORDS
    rd = _reference_readers(reference_root)
    m, f = epsocz_small(L=4, ntime=20, ngroup=10, lam=0.8, alpha=0.3)
    o = OracleChain(m, field=f, seed_words=SEED_WORDS, meas=True)
    o.init_expkv()
    o.init_g(1)
    half = m.ntime // 2
    mb = MeasurementBins(m, nbins=2, nmeas=1, output_addr=str(tmp_path) + "/")
    for b in range(2):   # two windows (a sweep between them): two bins of one measurement each
        if b:
            o.sweep(1, 1)
        rec = None
        for t in (half - 1, half, half + 1):
            rec = o.begin_measure(True, t, meas_number=1)
        mb.add(rec)
    mean = mb.finish()
    guide = str(tmp_path / "data" / "reading_guide.nml")
    basic = rd["read_namelist"](guide, "basic")
    obs = rd["read_obs_info"](guide)
    assert basic["total_width"] == mb.total_width and basic["n_bins"] == 2
    assert basic["field_width"] == m.lat.n_cell
    for e in mb.layout:
        assert obs[e["name"]]["offset_lo"] == e["offset_lo"] and obs[e["name"]]["offset_hi"] == e["offset_hi"]
        assert obs[e["name"]]["kind"] == e["kind"]
    data = np.fromfile(str(tmp_path / "data" / "out_core.bin"), dtype=np.float64)
    data = data.reshape((basic["total_width"], basic["n_bins"]), order="F")
    assert np.array_equal(data, mean)
    # the reference's post-processing recomputes every `_k` slot from its
    # r-space slot with a centred FFT (ifftshift / fftshift); its origin
    # differs from the one of Lat%k_phase (mod_meas.f90:546-566) by half the
    # lattice, which multiplies each k point by a fixed sign.  Check that the
    # recomputed slots equal the written ones up to one sign pattern over k,
    # the same for every field and bin.
    redone = rd["recalculate_k_data_function"](data.copy(), basic, obs)
    pattern = None
    for name in M.FIELD_NAMES:
        lo, hi = obs[name + "_k"]["offset_lo"], obs[name + "_k"]["offset_hi"]
        a, b = redone[lo - 1:hi], data[lo - 1:hi]
        assert np.allclose(np.abs(a), np.abs(b), rtol=1e-10, atol=1e-12), name
        big = np.abs(b) > 1e-8 * (1 + np.abs(b).max())
        sg = np.where(big, np.sign(a * b), 0.0)
        if pattern is None:
            pattern = np.zeros(sg.shape[0])
        for k in range(sg.shape[0]):
            for v in sg[k]:
                if v != 0:
                    assert pattern[k] in (0, v), (name, k)
                    pattern[k] = v
    assert np.count_nonzero(pattern) >= m.lat.n_cell // 2
