"""The exact round update of the mixed batch against FP64 numpy.

A scan round of the mixed batch decides its moves, then applies their
combined effect on G as one Woodbury update from the G the round started
from: W^-1 from an FP32 inverse refined by a Newton step with a
double-float residual, the products G(:,S) M and X Z on
the tensor cores with Ozaki-split BF16 operands whose per-level sums are
exact.  pqmc_exact_update_check runs exactly those kernels on a host G; the
reference is the sequence of rank-dim updates of update_phonon_field
(src/mod_update.f90:146-192) in FP64, one accepted move after another."""
import numpy as np
import pytest

from tests.helpers import rel_fro

pytestmark = pytest.mark.gpu

# The Ozaki products cut every operand row (column) into 5 pieces of 8 bits
# below its largest entry, so an entry of a product is exact to about 2^-40
# of (row max x column max x sqrt(inner dimension)); summed over the Ns^2
# entries of a round's update that is ~1e-10 of the update's Frobenius norm
# (FP32 arithmetic would leave ~1e-7).  The Newton-refined inverse is good to
# the square of the FP32 inverse's error.
UPDATE_TOL = 1e-9


def _sequential(g, sites, deltas):
    """The reference's accepted-move updates in order."""
    g = g.copy()
    ns = g.shape[0]
    for S, D in zip(sites, deltas):
        R = np.eye(len(S)) + g[np.ix_(S, S)] @ D
        T = D @ np.linalg.inv(R)
        E = np.zeros((len(S), ns), complex)
        E[np.arange(len(S)), S] = 1.0
        g = g + g[:, S] @ T @ (E - g[S, :])
    return g


def _case(ns, dim, nmoves, scale, seed):
    rng = np.random.default_rng(seed)
    # a G-like matrix: a projector of rank ns/2 plus a perturbation
    q, _ = np.linalg.qr(rng.normal(size=(ns, ns)) + 1j * rng.normal(size=(ns, ns)))
    g0 = q[:, : ns // 2] @ q[:, : ns // 2].conj().T
    g0 = g0 + 0.05 * (rng.normal(size=(ns, ns)) + 1j * rng.normal(size=(ns, ns)))
    sites = rng.permutation(ns)[: dim * nmoves].reshape(nmoves, dim)
    deltas = scale * (rng.normal(size=(nmoves, dim, dim)) + 1j * rng.normal(size=(nmoves, dim, dim)))
    return g0, sites, deltas


@pytest.mark.parametrize("ns,dim,nmoves,scale", [
    (392, 4, 16, 0.05),    # a full round of the 14x14 benchmark family (K = 64)
    (392, 4, 16, 0.5),     # large jumps
    (200, 4, 5, 0.1),      # K = 20: inner dimension padded to 32
    (130, 2, 13, 0.2),     # ragged row and column tiles (130 = 128 + 2)
    (77, 1, 40, 0.2),      # one site per move, one row tile
])
@pytest.mark.parametrize("flush_tile", [64, 32, 2, 1])
def test_exact_update_matches_sequential_fp64(ns, dim, nmoves, scale, flush_tile):
    from pqmc_allinone_gb300.engine import exact_update_check
    g0, sites, deltas = _case(ns, dim, nmoves, scale, seed=ns + dim + nmoves)
    want = _sequential(g0, sites, deltas)
    got = exact_update_check(g0, sites.reshape(-1), deltas, flush_tile)
    upd = np.linalg.norm(want - g0)
    err = np.linalg.norm(got - want)
    print(f"ns={ns} dim={dim} moves={nmoves} scale={scale} tile={flush_tile}: |err|/|update| {err / upd:.3e}, "
          f"|err|/|G| {err / np.linalg.norm(want):.3e}")
    assert err <= UPDATE_TOL * upd + 1e-14 * np.linalg.norm(want), (err, upd)
    # FP32-accurate arithmetic would leave ~1e-7 of the update: the test
    # resolves the difference
    assert err < 1e-6 * upd


@pytest.mark.parametrize("ns,dim,nmoves", [(392, 4, 16), (130, 2, 13), (77, 1, 40), (200, 4, 5)])
def test_pipelined_flush_bit_identical_to_quarter_stages(ns, dim, nmoves):
    """The pipeline (k_xflushp: X resident, Z's 32-column tiles streamed,
    two accumulator buffers) issues the products of k_xflush2 in the same
    order, stage by stage: the updated G is the same bit for bit, with one
    or two CTAs per row tile."""
    from pqmc_allinone_gb300.engine import exact_update_check
    g0, sites, deltas = _case(ns, dim, nmoves, 0.2, seed=3 * ns + nmoves)
    ref = exact_update_check(g0, sites.reshape(-1), deltas, 32)
    for ct in (2, 1):
        got = exact_update_check(g0, sites.reshape(-1), deltas, ct)
        assert np.array_equal(got, ref), ct


def test_exact_update_two_calls_and_zero_rows():
    """Two updates in a row from the same images (the slice images are
    reused between rounds and must not carry state), and a G with all-zero
    rows and columns (the zero grid of the slicing)."""
    from pqmc_allinone_gb300.engine import exact_update_check
    g0, sites, deltas = _case(160, 4, 12, 0.1, seed=5)
    g0[7, :] = 0.0
    g0[:, 11] = 0.0
    want1 = _sequential(g0, sites, deltas)
    got1 = exact_update_check(g0, sites.reshape(-1), deltas)
    assert rel_fro(got1, want1) < 1e-10
    s2 = sites[:3]
    want2 = _sequential(got1, s2, deltas[:3])
    got2 = exact_update_check(got1, s2.reshape(-1), deltas[:3])
    assert np.linalg.norm(got2 - want2) <= UPDATE_TOL * np.linalg.norm(want2 - got1) + 1e-14 * np.linalg.norm(want2)
