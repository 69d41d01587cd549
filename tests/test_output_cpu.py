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
    want = np.stack([recs[2 * b:2 * b + 2].real.mean(axis=0) for b in range(3)], axis=1)
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
    den = 3 + 2 * nc * M.FIELD_NAMES.index("den_den")
    assert np.array_equal(mean[:nc, 0], rec[den:den + nc].real)
    assert np.array_equal(mean[nc:2 * nc, 0], rec[den + nc:den + 2 * nc].real)
    assert mean[2 * nc, 0] == 2.0 and mean[2 * nc + 1, 0] == 0.0
    assert (tmp_path / "data" / "out_core5.bin").exists() and (tmp_path / "temp" / "tempout_core5.bin").exists()
    with pytest.raises(ValueError):
        reference_layout(m, [("a", "scalar"), ("a", "field")])
