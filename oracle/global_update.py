"""Oracle of the global moves: update_global / generate_newfield_global
(src/mod_update.f90:250-467) and the driver's global step
(src/Main_PQMC.f90:87-96), restated in numpy on top of the C++ oracle's
ran2 stream (oracle_rng_draw) and cal_new_weight_T0.

TEST INFRASTRUCTURE ONLY -- imported by tests/ to check the GPU results.  Parity status:
unpinned against reference outputs (the reference ships no golden vectors for
these moves); the restatement follows the cited lines draw by draw.

Two places where the reference's behaviour is undefined are made definite
here and in the library alike: the "kspace_time" range end
max(start_time + int(M/delt**2), ntime) (:326) is clipped to ntime (larger
values index beyond boson_field), and every move refreshes expKV on the
slices it changed (the "exchange" branch, :304-314, does not).
"""
from __future__ import annotations

import numpy as np

from oracle.oracle import rng_draw

SINGLE, EXCHANGE, KSPACE, KSPACE_TIME, ROTATE = 0, 1, 2, 3, 4
PI_SP = float(np.float32(np.pi))           # PI of nrtype is REAL(SP) (mod_nrtype.f90:42)


class Ran2:
    """ran2_s draws one at a time (rands, ran_sysm, irands of
    src/mod_ranstate.f90:221-236)."""

    def __init__(self, words):
        self.words = [int(w) for w in words]

    def rands(self) -> np.float32:
        r, self.words = rng_draw(self.words, 1)
        return r[0]

    def ran_sysm(self) -> np.float32:
        return np.float32(self.rands() * np.float32(2.0) - np.float32(1.0))

    def irands(self, n: int) -> int:
        k = int(np.float32(self.rands() * np.float32(n)))      # int(r*n), r*n in REAL(SP)
        return min(k, n - 1)


def _modi(i: int, n: int) -> int:
    return (i - 1) % n + 1


def generate(m, gp: dict, kind: int, rng: Ran2, field: np.ndarray):
    """generate_newfield_global (mod_update.f90:298-438) on a copy of field
    (n_bf, ntime).  Returns (new field, ph_ln_cw, t_first, t_last), times
    1-based."""
    f = np.array(field, dtype=np.float64, copy=True)
    nb, nt = f.shape
    D, M, dt, bias = m.D, m.M, m.spec.delt, m.spec.biased_phonon
    lncw = 0.0
    t0, t1 = 1, nt
    if kind == EXCHANGE:                                  # :304-314
        for _ in range(gp["n_global_update"]):
            a = rng.irands(nb)
            s = rng.irands(nb)
            f[[a, s], :] = f[[s, a], :]
    elif kind in (KSPACE, KSPACE_TIME):                   # :316-374
        kvec = np.array([2 * PI_SP * 0.5, 2 * PI_SP * 0.5])
        incell = [rng.irands(2) * 2.0 - 1.0 for _ in range(gp["bf_sets"])]
        # generate_newfield_space :441-467
        distance = 2 * gp["distance"] / gp["n_cell"]
        amplitude = distance * float(rng.rands())
        jump = np.zeros(nb)
        rpos = gp["cell_rpos"]                            # (n_cell, dim)
        for c in range(gp["n_cell"]):
            kr = 0.0
            for d in range(len(kvec)):
                kr += kvec[d] * rpos[c, d]
            for i in range(gp["bf_sets"]):
                jump[gp["bf_sets"] * c + i] = incell[i] * amplitude * np.cos(kr + 0.0)
        if kind == KSPACE_TIME:
            t0 = rng.irands(nt // 2) + 1
            t1 = min(max(t0 + int(1.0 * M / (dt * dt)), nt), nt)
        old = field
        f[:, t0 - 1:t1] = old[:, t0 - 1:t1] + jump[:, None]
        dE = 0.0
        for t in range(t0 - 1, t1):
            for b in range(nb):
                xn, xo = f[b, t], old[b, t]
                dE = dE + 0.5 * D * (xn * xn - xo * xo)
                dE = dE + (-bias * (xn - xo))
        if kind == KSPACE_TIME:
            kin = 0.5 * (M / (dt * dt))
            tm, tp = _modi(t0 - 1, nt) - 1, _modi(t1 + 1, nt) - 1
            for b in range(nb):
                a0, b0 = f[b, t0 - 1] - f[b, tm], old[b, t0 - 1] - old[b, tm]
                dE = dE + kin * (a0 * a0 - b0 * b0)
                a1, b1 = f[b, t1 - 1] - f[b, tp], old[b, t1 - 1] - old[b, tp]
                dE = dE + kin * (a1 * a1 - b1 * b1)
        lncw = lncw - dE * dt
    elif kind == ROTATE:                                  # :376-407
        ang = float(rng.ran_sysm()) * 0.1 * PI_SP
        r = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
        if rng.ran_sysm() < 0:
            r[:, 1] = -r[:, 1]
        for c in range(gp["n_cell"]):
            x, y = field[2 * c].copy(), field[2 * c + 1].copy()
            f[2 * c] = r[0, 0] * x + r[0, 1] * y
            f[2 * c + 1] = r[1, 0] * x + r[1, 1] * y
    elif kind == SINGLE:                                  # :408-432
        for _ in range(gp["n_global_update"]):
            u = rng.irands(nb)
            if gp["flip"]:
                tmp = -f[u]
            elif gp["shift"]:
                tmp = f[u] + float(rng.ran_sysm()) * gp["distance"]
            else:
                raise ValueError("single-bond move needs flip or shift")
            dE = 0.0
            if not gp["flip"]:
                s = 0.0
                for t in range(nt):
                    s += tmp[t] * tmp[t] - f[u, t] * f[u, t]
                dE = 0.5 * D * s
            s = 0.0
            for t in range(nt):
                s += -bias * (tmp[t] - f[u, t])
            dE = dE + s
            f[u] = tmp
            lncw = lncw - dE * dt
    else:
        raise ValueError(kind)
    return f, lncw, t0, t1


def prob(m, re_w: float) -> float:
    """cal_prob (mod_update.f90:475-500); only Re w enters."""
    R = np.exp(min(10.0, re_w))
    if m.spec.metropolis:
        p = min(1.0, R)
        return float(np.floor(p)) if m.spec.greatest_decent else p
    return R / (1 + R)


def update_global(oc, m, gp: dict, kind: int, ln_old: complex, rng: Ran2):
    """update_global(update_type) (mod_update.f90:250-292) on an
    OracleChain whose expKV matches its field.  Returns (accepted, ln_cw
    after the move).  The chain is left with the field of the outcome and
    its expKV."""
    old = oc.field()
    new, ph, _, _ = generate(m, gp, kind, rng, old)
    oc.set_field(new)
    oc.init_expkv()
    ln_new = oc.cal_new_weight()
    acc = float(rng.rands()) < prob(m, ln_new.real + ph - ln_old.real)
    if not acc:
        oc.set_field(old)
        oc.init_expkv()
        return False, ln_old
    return True, ln_new


def global_step(oc, m, gp: dict, loop: int, ln_cw: complex, words):
    """Main_PQMC.f90:87-96 before sweep `loop`.  Returns (accepted count,
    rng words after)."""
    rng = Ran2(words)
    forward = loop % 2 == 0
    if forward or (loop + 1) % gp["global_update_loop"] != 0:
        return 0, rng.words
    n = 0
    kinds = [KSPACE] + ([ROTATE] if gp["rotate"] else []) + [KSPACE_TIME]
    for k in kinds:
        a, ln_cw = update_global(oc, m, gp, k, ln_cw, rng)
        n += int(a)
    oc.set_rng(rng.words)
    if n > 0:
        oc.init_g(1)
    return n, rng.words
