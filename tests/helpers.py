"""Shared model builders and comparison helpers for the tests."""
import numpy as np

from pqmc_allinone_gb300 import model as M
from pqmc_allinone_gb300.rng import seed_words


def epsocz_small(L=4, ntime=40, ngroup=10, lam=0.8, alpha=0.0, jump=0.5, seed=1, bc=(0.0, 0.0)):
    spec = M.epsocz_spec(L, lam=lam, alpha=alpha, ntime=ntime, ngroup=ngroup, filling=0.5,
                         jump_distance=jump, bc_phase=bc)
    m = M.build_model(spec, twist_seed=7, twist=1e-3)
    f = M.field_gaussian(m, seed)
    return m, f


def general_bond_model(L=4, ntime=40, ngroup=10, lam=0.8, jump=0.5, seed=1):
    """Bond-modulated hopping t(1 - lam x_b) on a spinless square lattice,
    through get_expKV_general (expm): 2-site plaquettes with V = K."""
    kb = [0, 1, 1, 0]
    pfs = []
    for vert, off in ((False, (0, 0)), (False, (1, 0)), (True, (0, 0)), (True, (0, 1))):
        pfs.append(M.PfSpec(dim=2, n_cover=1.0, tsl=[2, 0, 1, 1], offset=list(off),
                            int_subsites=([0, 0, 1, 0, 1, 1] if vert else [0, 0, 1, 1, 0, 1]),
                            k_exist=True, v_exist=True, k_coe=1.0, kmat=[complex(v) for v in kb],
                            v_coe=1.0, vmat=[complex(v) for v in kb], bf_index=2 if vert else 1))
    sk = [0j] * 9
    for (i, j) in ((1, 2), (2, 1), (1, 3), (3, 1)):
        sk[(i - 1) + 3 * (j - 1)] = 1.0
    slater = M.PfSpec(dim=3, n_cover=3.0, tsl=[1, 0, 0, 1], offset=[0, 0],
                      int_subsites=[0, 0, 1, 1, 0, 1, 0, 1, 1], k_exist=True, v_exist=False,
                      k_coe=1.0, kmat=sk)
    spec = M.ModelSpec(lat_dim=2, n_subsite=1, lat_size=[L, L], lat_vec=[1, 0, 0, 1], site_vec=[0, 0],
                       periodic=[True, True], bc_phase=[0.0, 0.0], pfs=pfs, slater=slater, bf_sets=2,
                       model_name="GENERAL", delt=0.1, beta=ntime * 0.1, ngroup=ngroup, filling=0.5,
                       ep_parameter=lam, jump_distance=jump, tr_slater=False,
                       expkv_kind=M.EXPKV_GENERAL)
    m = M.build_model(spec, twist_seed=3, twist=1e-3)
    return m, M.field_gaussian(m, seed)


def epsoc_model(L=4, ntime=40, ngroup=10, lam=0.8, jump=0.5, seed=1):
    """EPSOC-type 2-site plaquettes through the get_expKV_epsoc closed form."""
    k = [0, 1, 1, 0]
    v = [0, 1j, -1j, 0]
    pfs = []
    for vert, off in ((False, (0, 0)), (False, (1, 0)), (True, (0, 0)), (True, (0, 1))):
        pfs.append(M.PfSpec(dim=2, n_cover=1.0, tsl=[2, 0, 1, 1], offset=list(off),
                            int_subsites=([0, 0, 1, 0, 1, 1] if vert else [0, 0, 1, 1, 0, 1]),
                            k_exist=True, v_exist=True, k_coe=1.0, kmat=[complex(x) for x in k],
                            v_coe=1.0, vmat=[complex(x) for x in v], bf_index=2 if vert else 1))
    sk = [0j] * 9
    for (i, j) in ((1, 2), (2, 1), (1, 3), (3, 1)):
        sk[(i - 1) + 3 * (j - 1)] = 1.0
    slater = M.PfSpec(dim=3, n_cover=3.0, tsl=[1, 0, 0, 1], offset=[0, 0],
                      int_subsites=[0, 0, 1, 1, 0, 1, 0, 1, 1], k_exist=True, v_exist=False,
                      k_coe=1.0, kmat=sk)
    spec = M.ModelSpec(lat_dim=2, n_subsite=1, lat_size=[L, L], lat_vec=[1, 0, 0, 1], site_vec=[0, 0],
                       periodic=[True, True], bc_phase=[0.0, 0.0], pfs=pfs, slater=slater, bf_sets=2,
                       model_name="EPSOC", delt=0.1, beta=ntime * 0.1, ngroup=ngroup, filling=0.5,
                       ep_parameter=lam, jump_distance=jump, tr_slater=False, tr_weight=True,
                       expkv_kind=M.EXPKV_EPSOC)
    m = M.build_model(spec, twist_seed=5, twist=1e-3)
    return m, M.field_gaussian(m, seed)


def rel_fro(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


SEED_WORDS = seed_words(42)
