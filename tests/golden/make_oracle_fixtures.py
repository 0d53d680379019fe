"""Record the oracle's output on the 1000 x 1000 FP64 workload (Philox seed 0).

    python tests/golden/make_oracle_fixtures.py

The oracle itself is pinned to the reference by ``make_golden.py``; this
fixture freezes its Philox-stream result (which the GPU must reproduce bit for
bit) so a different LAPACK build on another machine cannot move the target.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import id_error, interp_sid, rbrp_column_id  # noqa: E402
from robust_blockwise_random_pivoting_gb300 import workloads as W  # noqa: E402

if __name__ == "__main__":
    A = W.gaussian_exp()
    r = rbrp_column_id(A, 40, tol=1e-12, seed=0)
    T = interp_sid(A, r["perm"], r["k"])
    np.savez_compressed(os.path.join(HERE, "oracle_gexp1000_philox0.npz"), k=r["k"], perm=r["perm"],
                        ranks=r["ranks"], residuals=r["residuals"], draws=r["draws"],
                        id_err=id_error(A, r["perm"], T))
    print("k =", r["k"], "draws =", r["draws"])
