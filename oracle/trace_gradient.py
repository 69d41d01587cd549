"""FP64 Green's-function trace formula for the gradient of the projector
log-weight, evaluated directly on the CPU for small systems.

TEST INFRASTRUCTURE ONLY -- imported by tests/ to check the GPU adjoint
(pqmc_logweight_grad).  It shares no code with the device adjoint: the
propagators come from the oracle's own expKV tables and left/right_evolve,
G is formed by dense FP64 products without stabilisation (so it is meant for
short Lt, where B(Lt..1) stays well conditioned), and dE/dx is a Richardson-
extrapolated central difference of the oracle's get_expKV.

    W(x) = c Re log det(P^H B(Lt..1) P),   B(t) = E_{n_pf}(t) ... E_1(t),

with P the trial state, c = ncopy (x2 under TR_weight) as in
cal_new_weight_T0 (src/mod_evolution.f90:359-408; the weight of
src/mod_update.f90:104).  For the plaquette p of family f at slice t that
carries boson b, write the string as X E_p Y with X = P^H B(Lt..t+1)
E_{n_pf}(t)...E_{f+1}(t) and Y the rest of the family and everything to its
right applied to P.  Then

    dW/dx_{b,t} = c Re Tr[(X E_p Y)^-1 X dE_p Y]
                = c Re Tr[g dE_p E_p^-1],   g = R (X R)^-1 X,  R = E_f(t) ... P,

where g is the equal-time Green's function right after family f acts at
slice t (the g_h of src/mod_evolution.f90:330-357 at that point of the
string); only the plaquette's dim x dim block of g enters, because dE_p
touches its sites alone.  A boson that several plaquettes carry collects
every one of their terms.

Parity status: pinned against the oracle's own weight (value to 1e-12, every
gradient entry to its central finite difference, tests/test_trace_gradient_cpu.py);
like the oracle it builds on, unpinned against reference outputs, which the
reference does not ship.
"""
from __future__ import annotations

import numpy as np


def _dexp(o, kind: int, pf: int, pla: int, x: float, h: float = 1e-3) -> np.ndarray:
    """dE/dx of one plaquette propagator: Richardson extrapolation of two
    central differences (error O(h^4))."""
    def cd(hh):
        return (o.expkv_single(kind, pf, pla, x + hh, 0) - o.expkv_single(kind, pf, pla, x - hh, 0)) / (2.0 * hh)
    return (4.0 * cd(h / 2) - cd(h)) / 3.0


def logweight_grad_trace(m, field: np.ndarray, seed_words=None):
    """(W, grad, dets): the weight, grad[b, t] = dW/dx_{b,t} for the field
    (n_bf, ntime), and slogdet(P^H B P) as seen at every (slice, family)
    position (all equal in exact arithmetic; their spread checks the string)."""
    from oracle.oracle import OracleChain

    o = OracleChain(m, field=np.asarray(field, dtype=np.float64), seed_words=seed_words, meas=False)
    o.init_expkv()
    _, ekv_inv = o.expkv()
    npf, pd, mp, nt = len(m.pf), m.pdim, m.max_pla, m.ntime
    # flat (pdim, pdim, max_pla, n_pf, ntime), column-major
    ekv_inv = ekv_inv.reshape((pd, pd, mp, npf, nt), order="F")
    P = np.asarray(m.slater_q, dtype=np.complex128).reshape((m.ns, m.nelec), order="F")
    d = np.asarray(m.slater_d, dtype=np.complex128)

    # right factors R(t, f) = E_f(t) ... E_1(t) B(t-1..1) P, family 0 first
    R = {}
    r = P.copy(order="F")
    for t in range(1, nt + 1):
        for f in range(npf):
            r = o.left_evolve(t, f + 1, r)
            R[(t, f)] = r
    # left factors X(t, f) = P^H B(Lt..t+1) E_{n_pf}(t) ... E_{f+1}(t)
    grad = np.zeros((m.n_bf, nt))
    c = float(m.spec.ncopy) * (2.0 if m.spec.tr_weight else 1.0)
    dets = []
    x = P.conj().T.copy(order="F")
    for t in range(nt, 0, -1):
        for f in range(npf - 1, -1, -1):
            r = R[(t, f)]
            xr = x @ r
            dets.append(np.linalg.slogdet(xr))
            tab = m.pf[f]
            if m.spec.pfs[f].v_exist:
                g = r @ np.linalg.solve(xr, x)
                dim = tab.dim
                for p in range(tab.n_pla):
                    S = np.asarray(tab.site_list[p][:dim])
                    b = int(tab.bf_list[p])
                    xb = float(field[b, t - 1])
                    de = _dexp(o, m.expkv_kind, f, p, xb)
                    einv = ekv_inv[:dim, :dim, p, f, t - 1]
                    # Tr[g dE E^-1] over the plaquette's block of g
                    grad[b, t - 1] += c * np.real(np.trace(g[np.ix_(S, S)] @ (de @ einv)))
            x = o.right_evolve(t, f + 1, x)
    sign, logabs = dets[-1]
    lndet = logabs + np.log(sign) + 2.0 * np.sum(np.log(d))
    W = c * np.real(lndet)
    return W, grad, dets


def logweight_grad_trace_stable(m, field: np.ndarray, seed_words=None, block: int | None = None):
    """grad[b, t] = dW/dx_{b,t} by the same trace formula, stabilised for long
    Lt: the right factor R and the left factor X are re-orthonormalised after
    every slice (g = R (X R)^-1 X does not change when R is multiplied on the
    right, or X on the left, by an invertible matrix), the right factors are
    kept only at the first slice of every block of `block` slices (ngroup by
    default) and rebuilt inside a block as the left factor passes through
    it.  Memory: Lt/block + block*n_pf matrices of Ns x nelec."""
    from oracle.oracle import OracleChain

    o = OracleChain(m, field=np.asarray(field, dtype=np.float64), seed_words=seed_words, meas=False)
    o.init_expkv()
    _, ekv_inv = o.expkv()
    npf, pd, mp, nt = len(m.pf), m.pdim, m.max_pla, m.ntime
    ekv_inv = ekv_inv.reshape((pd, pd, mp, npf, nt), order="F")
    P = np.asarray(m.slater_q, dtype=np.complex128).reshape((m.ns, m.nelec), order="F")
    nb = int(block or m.ngroup)
    c = float(m.spec.ncopy) * (2.0 if m.spec.tr_weight else 1.0)

    def orth_cols(a):
        return np.asfortranarray(np.linalg.qr(a)[0])

    def orth_rows(a):
        return np.asfortranarray(np.linalg.qr(a.conj().T)[0].conj().T)

    ck = {}
    r = orth_cols(P)
    for t in range(1, nt + 1):
        if (t - 1) % nb == 0:
            ck[t] = r.copy(order="F")
        for f in range(npf):
            r = o.left_evolve(t, f + 1, r)
        r = orth_cols(r)
    grad = np.zeros((m.n_bf, nt))
    x = orth_rows(P.conj().T)
    for t0 in sorted(ck, reverse=True):
        t1 = min(t0 + nb - 1, nt)
        R = {}
        r = ck[t0]
        for t in range(t0, t1 + 1):
            for f in range(npf):
                r = o.left_evolve(t, f + 1, r)
                R[(t, f)] = r
            r = orth_cols(r)
        for t in range(t1, t0 - 1, -1):
            for f in range(npf - 1, -1, -1):
                tab = m.pf[f]
                if m.spec.pfs[f].v_exist:
                    r = R[(t, f)]
                    y = np.linalg.solve(x @ r, x)   # g = r y
                    dim = tab.dim
                    for p in range(tab.n_pla):
                        S = np.asarray(tab.site_list[p][:dim])
                        b = int(tab.bf_list[p])
                        de = _dexp(o, m.expkv_kind, f, p, float(field[b, t - 1]))
                        einv = ekv_inv[:dim, :dim, p, f, t - 1]
                        gb = r[S, :] @ y[:, S]
                        grad[b, t - 1] += c * np.real(np.trace(gb @ (de @ einv)))
                x = o.right_evolve(t, f + 1, x)
            x = orth_rows(x)
    return grad
