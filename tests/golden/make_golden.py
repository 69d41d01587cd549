"""Generate the committed golden fixtures under tests/golden/.

The reference has no test vectors of its own and cannot be built here, so
the fixtures are produced by the CPU oracle (oracle/pqmc_oracle.cpp, a
line-cited FP64 restatement) and pin it, and the GPU path, against
regressions:

* ran2_seed42.npy / ran2_seed122.npy -- the first 4096 ran2 draws after
  init_rng_by_seed(42) / (122) (src/mod_ranstate.f90:171-191, 267-283);
* sweep_epsocz4.npz -- a 4x4 EPSOCZ chain (Lt=40, ngroup=10, lambda=0.8,
  seeded field) after init_g_T0 and after 3 sweeps: G, field, ln_cw,
  accept counts and ran2 words.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import OracleChain, rng_draw  # noqa: E402
from pqmc_allinone_gb300.rng import seed_words  # noqa: E402
from tests.helpers import epsocz_small  # noqa: E402


def main():
    for seed in (42, 122):
        draws, _ = rng_draw(seed_words(seed), 4096)
        np.save(os.path.join(HERE, f"ran2_seed{seed}.npy"), draws)
    m, f = epsocz_small(L=4, ntime=40, ngroup=10, lam=0.8)
    o = OracleChain(m, field=f, seed_words=seed_words(42))
    o.init_expkv()
    o.init_g(1)
    g0, s0 = o.g(), o.state()
    o.sweep(1, 3)
    s3 = o.state()
    np.savez_compressed(
        os.path.join(HERE, "sweep_epsocz4.npz"),
        field0=f, g0=g0, lncw0=np.array(s0["ln_cw"]), g3=o.g(), field3=o.field(),
        lncw3=np.array(s3["ln_cw"]), acc3=np.array([s3["positive_accept"], s3["negative_accept"]]),
        rng3=np.array(s3["rng"], dtype=np.int64))
    print("golden fixtures written")


if __name__ == "__main__":
    main()
