"""Generate the golden fixtures that pin the CPU oracle to the reference.

Run in a container that has the reference checkout (read-only):

    python tests/golden/make_golden.py REFERENCE_ROOT

It executes the reference's own Python RBRP (``python/RBRP.ipynb`` code cells
2, 7 and 11) from REFERENCE_ROOT into a private namespace and records its
outputs on seeded inputs.  Two single-line corrections are applied to the
executed text of cell 11, and nothing else:

* ``aux = row_perm[i:i+block_size]`` -> ``... .copy()`` (the view bug in the
  block swap, cell 11 line 126);
* ``diags[row_perm[i+1:]]`` -> ``diags[row_perm[i:]]`` in the zero-residual
  stop test (cell 11 line 164).

Run inputs are zero-prefixed (``workloads.zero_prefixed``) so that no sampled
position ever falls inside the block being filled; on such inputs the
corrected notebook and the ``setdiff``-based swap of ``matlab/RBRP.m`` agree,
so the fixtures pin the oracle's arithmetic with the reference's own rng
(PCG64, seed 42).  The unpatched notebook is run once more on the 1000 x 1000
workload to record the effect of the swap bug.

Outputs (``tests/golden/*.npz``) are small and are read by ``tests/``; the
reference itself is never read at test time.
"""
import json
import os
import sys
import time
import warnings

import numpy as np
import scipy.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from robust_blockwise_random_pivoting_gb300 import workloads as W  # noqa: E402

PATCHES = [
    ("aux = row_perm[i:i+block_size]\n", "aux = row_perm[i:i+block_size].copy()\n"),
    ("np.count_nonzero(diags[row_perm[i+1:]]) < 1):\n            L = L[:,:i]",
     "np.count_nonzero(diags[row_perm[i:]]) < 1):\n            L = L[:,:i]"),
]


def load_reference(root, patched=True):
    nb = json.load(open(os.path.join(root, "python", "RBRP.ipynb")))
    cells = nb["cells"]
    ns = dict(np=np, spla=spla, time=time, warnings=warnings, SEED=42, TOL_FP=1e-12)
    for c in (2, 7, 11):
        src = "".join(cells[c]["source"])
        if c == 11 and patched:
            for old, new in PATCHES:
                assert src.count(old) == 1, old
                src = src.replace(old, new)
        exec(compile(src, f"RBRP.ipynb#c{c}", "exec"), ns)
    return ns


def sampler_cases(n_cases=200):
    """numpy Generator(Philox(key=seed)).choice(N, size, p, replace=False) outputs."""
    rng = np.random.default_rng(7)
    out = []
    for case in range(n_cases):
        N = int(rng.integers(1, 400))
        kind = case % 4
        if kind == 0:
            w = rng.random(N)
        elif kind == 1:
            w = rng.random(N) ** 8                      # concentrated: several rounds
        elif kind == 2:
            w = rng.random(N) * (rng.random(N) < 0.3)  # many zeros
        else:
            w = np.exp(-rng.random(N) * 40)             # wide dynamic range
        nnz = int(np.count_nonzero(w))
        if nnz == 0:
            w[0] = 1.0
            nnz = 1
        size = int(min(rng.integers(1, 65), nnz))
        seed = int(rng.integers(0, 2**32))
        g = np.random.Generator(np.random.Philox(key=seed))
        idx = g.choice(N, size=size, p=w / sum(w), replace=False)
        draws_probe = np.random.Generator(np.random.Philox(key=seed))
        # number of uniforms consumed: position of the generator after choice
        st_after = g.bit_generator.state
        out.append(dict(w=w, size=size, seed=seed, idx=np.asarray(idx, np.int64),
                        state_counter=np.array(st_after["state"]["counter"], np.uint64),
                        buffer_pos=int(st_after["buffer_pos"])))
        del draws_probe
    return out


def filter_cases(ns):
    rng = np.random.default_rng(11)
    Rs, tols, outs = [], [], []
    for case in range(120):
        b = int(rng.integers(1, 65))
        rows = int(rng.integers(1, b + 1)) if case % 5 == 0 else b
        R = np.triu(rng.standard_normal((rows, b)))
        decay = np.exp(-rng.random() * 30 * np.arange(rows) / max(rows, 1))
        R = R * decay[:, None]
        if case % 7 == 0 and rows > 2:
            R[rows // 2:] = 0.0                      # exact rank deficiency
        tol = [1.0 / b, 1e-3, 0.5, 1e-12][case % 4]
        Rs.append(R)
        tols.append(tol)
        outs.append(int(ns["_block_size_local_clip"](R, tol)))
    return Rs, tols, outs


def rpid_cases(ns):
    """Patched notebook blocked_rpid on zero-prefixed inputs (rows = items)."""
    specs = [
        ("gexp", W.zero_prefixed(W.gaussian_exp(60, 150, decay=6.0, seed=1), 64), 8, 1e-10),
        ("snn", W.zero_prefixed(W.snn(80, 160, r=60, r1=10, density=0.1, seed=2), 72), 6, 1e-12),
        ("gmm", W.zero_prefixed(W.gmm(40, 300, nclusters=8, seed=3)[0], 48), 5, 1e-4),
        ("gexp_b1tol", W.zero_prefixed(W.gaussian_exp(50, 90, decay=4.0, seed=4), 60), 12, None),
    ]
    res = {}
    for name, A, b, tol in specs:
        X = A.T.copy()
        kmax = min(A.shape)
        row_perm, L, residuals, time_pivot, ranks = ns["blocked_rpid"](
            X, kmax, b=b, tol=tol, mode="rp", ortho=1)
        k = int(ranks[-1])
        Wsub, _ = ns["interpolation"](X, row_perm, k, mode="sid")
        err = ns["id_error"](X, row_perm, Wsub) / spla.norm(X, ord="fro") ** 2
        res[name] = dict(A=A, b=b, tol=(-1.0 if tol is None else tol), row_perm=row_perm,
                         L=L, residuals=residuals, ranks=ranks, W=Wsub, err=err)
    return res


def main(root):
    ns = load_reference(root, patched=True)
    cases = sampler_cases()
    np.savez_compressed(
        os.path.join(HERE, "sampler_numpy_choice.npz"),
        n=len(cases),
        w=np.concatenate([c["w"] for c in cases]),
        wlen=np.array([c["w"].size for c in cases]),
        size=np.array([c["size"] for c in cases]),
        seed=np.array([c["seed"] for c in cases], dtype=np.uint64),
        idx=np.concatenate([c["idx"] for c in cases]),
        counter=np.stack([c["state_counter"] for c in cases]),
        buffer_pos=np.array([c["buffer_pos"] for c in cases]),
    )
    Rs, tols, outs = filter_cases(ns)
    np.savez_compressed(
        os.path.join(HERE, "filter_local_clip.npz"),
        R=np.concatenate([r.ravel() for r in Rs]),
        shape=np.array([r.shape for r in Rs]), tol=np.array(tols), bs=np.array(outs))
    res = rpid_cases(ns)
    flat = {}
    for name, d in res.items():
        for key, val in d.items():
            flat[f"{name}__{key}"] = np.asarray(val)
    np.savez_compressed(os.path.join(HERE, "blocked_rpid_patched.npz"), names=np.array(list(res)), **flat)

    # the unpatched reference on the 1000 x 1000 workload: record the swap bug
    ns0 = load_reference(root, patched=False)
    A = W.gaussian_exp()
    rp, L, residuals, tp, ranks = ns0["blocked_rpid"](A.T.copy(), 1000, b=40, tol=1e-12, mode="rp", ortho=1)
    k = int(ranks[-1])
    np.savez_compressed(os.path.join(HERE, "blocked_rpid_unpatched_gexp1000.npz"),
                        k=k, unique_in_S=len(set(rp[:k].tolist())),
                        is_permutation=len(set(rp.tolist())) == rp.size, residuals=residuals)
    print("fixtures written; unpatched notebook on gexp1000: k =", k,
          "unique =", len(set(rp[:k].tolist())))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_ROOT (the reference checkout, read-only)")
    main(sys.argv[1])
