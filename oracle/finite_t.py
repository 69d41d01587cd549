"""FP64 finite-temperature Green's function and weight on the CPU: the
FTQMC branch of src/mod_evolution.f90:409-785 (init_g_FT, cal_g_and_det_FT,
get_g_scratch_FT, cal_new_weight_FT), restated with numpy on top of the
oracle's one-way propagators (OracleChain.left_evolve / right_evolve).

TEST INFRASTRUCTURE ONLY -- imported by tests/ to check the GPU finite-T
path.  The reference marks this branch "not used for now" (:409) and leaves
it unfinished; the restatement follows its algorithm with three corrections,
each a departure from the reference's text:

  * init_g_FT (:411-489) ends with cal_g_and_det_FT(rmat^H, rmat,
    D(nblock-1), D(nblock-1), R(nblock-1)^H, R(nblock-1)), i.e. it forms
    (1 + B B^H)^-1 from the right string alone.  At the end of the forward
    propagation the left string is B(beta, beta) = 1, held by block nblock
    (Q = R = 1, D = 1, set at :427-434), so the call here takes block nblock
    as the left factors and block nblock-1 as the right ones.
  * get_g_scratch_FT backward (:700-720) decomposes the left product
    D Q B(slices) = U S V^H and stores Q := U, R := R V^H, which swaps the
    roles of the two unitary factors in B(beta, tau) = R_l D_l Q_l.  Here
    the unitary factor goes to Q_l and the rest to R_l.
  * cal_new_weight_FT (:748-785) scales rmat(:, i) by the whole D vector
    (`rmat(:, i) * d_temp`); here column i is scaled by d_temp(i), as in
    init_g_FT (:463-465).
  * The strings are decomposed by QR with column pivoting (LAPACK zgeqp3
    through scipy; A P = Q R, D = |diag R|, V = D^-1 R P^T), not by the
    singular value decomposition udv of :470, 684, 711, 773.  The product
    B Q D whose decomposition carries the string is graded by columns, and
    the SVD (zgesvd / zgesdd) is accurate only to eps times its largest
    singular value, so the small scales are lost: on the free-fermion
    check below the SVD strings put Re ln det off by 0.03 at beta = 8 and
    G off by O(1) at beta = 12, while the pivoted QR stays within 1e-12 to
    beta = 100.  The decomposition of the scale-separated middle matrix in
    cal_g_and_det_FT (:577) keeps the SVD.

Conventions (the reference's): the right string of block b is
B(t_b, 0) = Q_r D_r R_r, t_b = ngroup (b - 1); the left string of block b+1
is B(beta, t_b) = R_l D_l Q_l; g = (1 + B(t,0) B(beta,t))^-1 and
g_h = 1 - g (:614-618), ln_cw = log det(1 + B(beta, 0)) (x2 Re under
TR_weight, x ncopy, Im reduced to the principal branch, :621-626).  udv is
the singular value decomposition (zudv, src/mod_matrixlib.f90:704-743):
A = U S V^H with A overwritten by U (kept for the middle matrix of
cal_g_and_det_FT; the strings use the pivoted QR above).  Blocks are 1-based as in the
reference; nblock = ntime / ngroup + 2 and ntime must be a multiple of
ngroup.

Parity status: unpinned against reference outputs (the branch is unused
and unfinished upstream); pinned instead by the dense known answer
(1 + B(beta,0))^-1 at short beta, the free-fermion (lambda = 0) answer by
eigen-decomposition of the slice propagator at long beta, and the err_fast
invariant of the fast update against this scratch (tests/test_finite_t_cpu.py).
"""
from __future__ import annotations

import numpy as np


def udv(a: np.ndarray):
    """A = U diag(S) V^H (zudv, src/mod_matrixlib.f90:704-743)."""
    u, s, vh = np.linalg.svd(a)
    return u, s.astype(np.complex128), vh


def udv_strings(a: np.ndarray):
    """A = Q diag(D) V by QR with column pivoting: A P = Q R, D = |diag R|,
    V = D^-1 R P^T (well conditioned; D keeps every scale of a graded A)."""
    import scipy.linalg as sl
    q, r, piv = sl.qr(a, pivoting=True)
    d = np.abs(np.diag(r))
    v = np.zeros_like(r)
    v[:, piv] = r / d[:, None]
    return q, d.astype(np.complex128), v


def _slices_forward(o, x, t_from, t_to):
    """B(t_to) ... B(t_from) x: left_evolve over families 1..n_pf per slice
    (init_g_FT :451-456)."""
    npf = len(o.m.pf)
    for p in range(t_from, t_to + 1):
        for pf in range(1, npf + 1):
            x = o.left_evolve(p, pf, x)
    return x


def _slices_backward(o, y, t_hi, t_lo):
    """y B(t_hi) ... B(t_lo): right_evolve over families n_pf..1 per slice
    (get_g_scratch_FT :704-708)."""
    npf = len(o.m.pf)
    for p in range(t_hi, t_lo - 1, -1):
        for pf in range(npf, 0, -1):
            y = o.right_evolve(p, pf, y)
    return y


# 2*pi with pi of nrtype's single-precision kind, as the reference reduces
# the branch (cmplx(real(z), mod(aimag(z), 2*pi)), :626)
TWO_PI_SP = 2.0 * float(np.float32(np.pi))


def _principal(ln: complex) -> complex:
    return complex(ln.real, float(np.fmod(ln.imag, TWO_PI_SP)))


def cal_g_and_det_ft(m, q_l, q_r, d_l, d_r, r_l, r_r, cal_g=True):
    """g_h and ln_cw from B(t,0) = Q_r D_r R_r and B(beta,t) = R_l D_l Q_l
    (cal_g_and_det_FT, src/mod_evolution.f90:491-628): the scales split at
    1 (:527-545), QDR = Dr_gt^-1 (Q_l Q_r)^-1 Dl_gt^-1 + Dr_lt R_r R_l Dl_lt
    (:549-570), its udv (:577), ln_cw (:580-581) and
    g = Q_l^-1 Dl_gt^-1 V D^-1 U^H Dr_gt^-1 Q_r^-1 (:594-618)."""
    ns = q_r.shape[0]
    big_l = np.abs(d_l) > 1.0
    big_r = np.abs(d_r) > 1.0
    dl_gt = np.where(big_l, d_l, 1.0 + 0j)
    dl_lt = np.where(big_l, 1.0 + 0j, d_l)
    dr_gt = np.where(big_r, d_r, 1.0 + 0j)
    dr_lt = np.where(big_r, 1.0 + 0j, d_r)
    qlqr = q_r.conj().T @ q_l.conj().T                      # (Q_l Q_r)^-1
    rr_rl = r_r @ r_l
    qdr = rr_rl * dr_lt[:, None] * dl_lt[None, :] + qlqr / dr_gt[:, None] / dl_gt[None, :]
    u, s, vh = udv(qdr)
    ln = (np.log(np.linalg.det(q_l)) + np.log(np.linalg.det(q_r)) + np.sum(np.log(s))
          + np.sum(np.log(dl_gt)) + np.sum(np.log(dr_gt)) + np.log(np.linalg.det(u))
          + np.log(np.linalg.det(vh)))
    g_h = None
    if cal_g:
        # Q_l^-1 Dl_gt^-1 (V^H)^-1 S^-1 U^-1 Dr_gt^-1 Q_r^-1
        r_ql = (q_l.conj().T / dl_gt[None, :]) @ vh.conj().T
        r_ql = r_ql / s[None, :]
        qr_q = u.conj().T @ (q_r.conj().T / dr_gt[:, None])
        g = r_ql @ qr_q
        g_h = np.eye(ns, dtype=np.complex128) - g
    if m.spec.tr_weight:
        ln = ln + np.conj(ln)
    ln = ln * m.spec.ncopy
    return g_h, _principal(complex(ln))


class FiniteT:
    """Finite-temperature Q/D/R strings and G of one oracle chain."""

    def __init__(self, o):
        self.o = o
        m = o.m
        self.m = m
        if m.ntime % m.ngroup != 0:
            raise ValueError("ntime must be a multiple of ngroup")
        self.ns = m.ns
        self.nblock = m.ntime // m.ngroup + 2
        eye = np.eye(self.ns, dtype=np.complex128)
        self.q = [eye.copy() for _ in range(self.nblock + 1)]   # index 1..nblock
        self.d = [np.ones(self.ns, dtype=np.complex128) for _ in range(self.nblock + 1)]
        self.r = [eye.copy() for _ in range(self.nblock + 1)]
        self.g_h = None
        self.ln_cw = 0j
        self.err_fast_max = 0.0

    def _right_step(self, blk_old, blk_new, t_from, t_to, store=True):
        """Propagate the right string of block blk_old through slices
        t_from..t_to, scale by its D, udv (init_g_FT :450-475)."""
        x = _slices_forward(self.o, self.q[blk_old].copy(), t_from, t_to)
        x = x * self.d[blk_old][None, :]
        u, s, v = udv_strings(x)
        q, d, r = u, s, v @ self.r[blk_old]
        if store:
            self.q[blk_new], self.d[blk_new], self.r[blk_new] = q, d, r
        return q, d, r

    def _left_step(self, blk_old, blk_new, t_hi, t_lo):
        """Propagate the left string of block blk_old (B(beta,t) = R D Q)
        back through slices t_hi..t_lo, scale rows by its D and decompose:
        Y = D Q B(slices), Y^H = Q' D' V', so Y = V'^H D' Q'^H and
        Q_l := Q'^H, R_l := R_old V'^H (get_g_scratch_FT :700-720, with the
        unitary factor on the right where B(beta,t) = R_l D_l Q_l wants it)."""
        y = _slices_backward(self.o, self.q[blk_old].copy(), t_hi, t_lo)
        y = self.d[blk_old][:, None] * y
        q, s, v = udv_strings(y.conj().T)
        self.q[blk_new], self.d[blk_new], self.r[blk_new] = q.conj().T, s, self.r[blk_old] @ v.conj().T

    def init_g(self, start_time: int = 1):
        """init_g_FT(start_time), src/mod_evolution.f90:411-489 (corrected
        final call)."""
        m = self.m
        eye = np.eye(self.ns, dtype=np.complex128)
        for b in (1, self.nblock):
            self.q[b], self.d[b], self.r[b] = eye.copy(), np.ones(self.ns, np.complex128), eye.copy()
        start_block = start_time // m.ngroup + 1
        start_by_block = (start_block - 1) * m.ngroup + 1
        if start_by_block > start_time:
            raise ValueError("start_time_by_block > start_time")
        for p0 in range(start_by_block, m.ntime + 1, m.ngroup):
            blk = (p0 + m.ngroup - 1 - 1) // m.ngroup + 2
            self._right_step(blk - 1, blk, p0, p0 + m.ngroup - 1)
        nb = self.nblock
        self.g_h, self.ln_cw = cal_g_and_det_ft(m, self.q[nb], self.q[nb - 1], self.d[nb], self.d[nb - 1],
                                                self.r[nb], self.r[nb - 1])
        return self.g_h, self.ln_cw

    def get_g_scratch(self, time: int, forward: bool, g_fast=None, ln_fast=None):
        """get_g_scratch_FT(time, forward, loop), src/mod_evolution.f90:631-745
        (corrected left-string roles).  Returns (err_g, err_lnw) against the
        fast-updated G and ln_cw when given."""
        m = self.m
        if forward:
            blk = time // m.ngroup + 1
            self._right_step(blk - 1, blk, time - m.ngroup, time - 1)
            l_b, r_b = blk + 1, blk
        else:
            blk = time // m.ngroup + 2
            if m.ngroup == 1:
                blk -= 1
            self._left_step(blk + 1, blk, time + m.ngroup - 1, time)
            l_b, r_b = blk, blk - 1
        g_h, ln = cal_g_and_det_ft(m, self.q[l_b], self.q[r_b], self.d[l_b], self.d[r_b],
                                   self.r[l_b], self.r[r_b])
        e_g = float(np.max(np.abs(g_fast - g_h))) if g_fast is not None else 0.0
        e_w = abs((ln - ln_fast).real) if ln_fast is not None else 0.0
        self.err_fast_max = max(self.err_fast_max, e_g, e_w)
        self.g_h, self.ln_cw = g_h, ln
        return e_g, e_w

    def cal_new_weight(self) -> complex:
        """cal_new_weight_FT, src/mod_evolution.f90:748-785 (columns scaled by
        their own D entry); the strings are left intact."""
        m = self.m
        q, d, r = self.q[1].copy(), self.d[1].copy(), self.r[1].copy()
        for p0 in range(1, m.ntime + 1, m.ngroup):
            x = _slices_forward(self.o, q, p0, p0 + m.ngroup - 1) * d[None, :]
            u, s, v = udv_strings(x)
            q, d, r = u, s, v @ r
        nb = self.nblock
        _, ln = cal_g_and_det_ft(m, self.q[nb], q, self.d[nb], d, self.r[nb], r, cal_g=False)
        return ln


def dense_b(o, t_lo: int = 1, t_hi: int | None = None) -> np.ndarray:
    """B(t_hi, t_lo - 1) = B(t_hi) ... B(t_lo) as one dense product (no
    stabilisation: for short beta only)."""
    m = o.m
    t_hi = m.ntime if t_hi is None else t_hi
    return _slices_forward(o, np.eye(m.ns, dtype=np.complex128), t_lo, t_hi)


def dense_g_and_weight(o) -> tuple[np.ndarray, complex]:
    """The known answer at short beta: g_h = 1 - (1 + B(beta,0))^-1 and
    ln_cw = ncopy log det(1 + B(beta,0)) (x2 Re under TR_weight)."""
    m = o.m
    b = dense_b(o)
    a = np.eye(m.ns, dtype=np.complex128) + b
    g_h = np.eye(m.ns, dtype=np.complex128) - np.linalg.inv(a)
    sign, lad = np.linalg.slogdet(a)
    ln = complex(lad, np.angle(sign))
    if m.spec.tr_weight:
        ln = ln + np.conj(ln)
    return g_h, _principal(ln * m.spec.ncopy)


def free_fermion_g(o) -> tuple[np.ndarray, float]:
    """The known answer at any beta for a field-independent propagator
    (lambda = 0): B(beta,0) = Bs^ntime with Bs = B(1) diagonalisable,
    Bs = V diag(w) V^-1, so g_h = V diag(w^n / (1 + w^n)) V^-1 and
    Re ln det(1 + B) = sum Re log(1 + w^n), evaluated without forming w^n
    for the large eigenvalues."""
    m = o.m
    bs = dense_b(o, 1, 1)
    w, v = np.linalg.eig(bs)
    n = m.ntime
    lw = n * np.log(w.astype(np.complex128))        # log w^n
    # w^n / (1 + w^n) = 1 / (1 + w^-n), stable for |w| > 1 and < 1 alike
    frac = np.where(lw.real > 0, 1.0 / (1.0 + np.exp(-lw)), np.exp(lw) / (1.0 + np.exp(lw)))
    g_h = (v * frac[None, :]) @ np.linalg.inv(v)
    re = float(np.sum(np.where(lw.real > 0, lw.real + np.log(np.abs(1.0 + np.exp(-lw))),
                               np.log(np.abs(1.0 + np.exp(lw))))))
    c = m.spec.ncopy * (2 if m.spec.tr_weight else 1)
    return g_h, c * re
