"""Field files in the reference's import_ph_field layout (Main_PQMC.f90:
355-369: ntime records of n_bf values, Fortran F18.6) and the checkpoint
container; no GPU needed."""
import numpy as np
import pytest

from pqmc_allinone_gb300 import checkpoint as ck
from tests.helpers import epsocz_small


def test_f18_6_layout(tmp_path):
    f = np.array([[0.5, -1.25], [1234567.1234564, -0.0000004], [3.0, 1e-7]])   # (n_bf=3, ntime=2)
    p = tmp_path / ck.FIELD_FILE
    ck.write_ph_field(str(p), f)
    lines = p.read_text().splitlines()
    assert len(lines) == 2 and all(len(x) == 3 * 18 for x in lines)
    assert lines[0] == "          0.500000    1234567.123456          3.000000"
    assert lines[1] == "         -1.250000         -0.000000          0.000000"


def test_field_file_round_trip(tmp_path):
    m, f = epsocz_small(L=4, ntime=20)
    p = tmp_path / ck.FIELD_FILE
    ck.write_ph_field(str(p), f)
    g = ck.read_ph_field(str(p), m.n_bf, m.ntime)
    assert g.shape == f.shape
    assert np.max(np.abs(g - f)) <= 5e-7
    assert np.array_equal(g, np.round(f, 6))


def test_field_file_errors(tmp_path):
    p = tmp_path / "short.dat"
    ck.write_ph_field(str(p), np.zeros((4, 3)))
    with pytest.raises(ValueError):
        ck.read_ph_field(str(p), 4, 5)          # too few records
    with pytest.raises(ValueError):
        ck.read_ph_field(str(p), 5, 3)          # records too short
    q = tmp_path / "wide.dat"
    ck.write_ph_field(str(q), np.array([[1e12]]))
    with pytest.raises(ValueError):
        ck.read_ph_field(str(q), 1, 1)          # F18.6 overflow written as asterisks


class _FakeChain:
    def __init__(self, m, f, i):
        self.m, self._f, self.i = m, f, i

    def field(self):
        return self._f

    def state(self):
        return {"rng": [1 + self.i, -2, 3, -4, 5], "positive_accept": 10 + self.i, "negative_accept": 20,
                "err_fast_max": 1e-9, "err_fast": 2e-10, "err_g": 3e-11, "err_g_rel_max": 4e-6,
                "ln_cw": complex(123.5, -0.25)}


def test_checkpoint_round_trip(tmp_path):
    ms = [epsocz_small(L=4, ntime=20, seed=s) for s in (1, 2)] + [epsocz_small(L=6, ntime=40, seed=3)]
    chains = [_FakeChain(m, f, i) for i, (m, f) in enumerate(ms)]
    p = str(tmp_path / "ck.npz")
    with pytest.raises(ValueError):
        ck.save_checkpoint(p, chains, 3)        # only after an even (forward) sweep
    ck.save_checkpoint(p, chains, 4)
    d = ck.load_checkpoint(p)
    assert d["loop"] == 4 and len(d["chains"]) == 3
    for c, s in zip(chains, d["chains"]):
        assert np.array_equal(s["field"], c.field())
        assert s["state"] == c.state()
    ck._check_geometry(d, [m for m, _ in ms])
    with pytest.raises(ValueError):
        ck._check_geometry(d, [ms[0][0], ms[0][0], ms[0][0]])
