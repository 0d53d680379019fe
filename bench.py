#!/usr/bin/env python
"""Benchmark of the GB300 adaptive RBRP column ID (one JSON line on stdout).

Default workload ``blocks4096`` (batched): 4096 off-diagonal blocks of a
Gaussian kernel k(x, y) = exp(-|x - y|^2 / (2 * 0.5^2)) between clusters of
3-D points uniform in unit cubes whose centres are 2 to 8 apart, m and n
log-uniform in [64, 2048], FP32 storage (each block scaled by its largest
entry, which a column ID is invariant to), squared relative tolerance 1e-8
(relative Frobenius 1e-4), block size b chosen by the library's autotuner,
Philox key = rank * 4096 + problem.  A step is one persistent launch (a CUDA
graph) that computes all 4096 IDs (S, T, k, error estimate), so ``value`` is
matrices/s.  The inputs (5.4 GB) are larger than L2: no flush is needed.
The plain FP64 and FP32 one-launch-per-matrix forms are timed on a seeded
random subset of 64 of the same blocks, and the 16384^2 single-matrix ID
time of the ``snn16k`` workload is reported beside the line.

Single-matrix workloads (``--workload snn16k`` ...): the sparse non-negative
low-rank-plus-tail matrix A = sum_{j<=100} (10/j) x_j y_j^T + sum_{100<j<=2000}
(1/j) x_j y_j^T, x_j, y_j i.i.d. with density 0.02 and Uniform[0,1] nonzeros,
stored dense FP32 (FP64 copy for the plain form and the error check); b = 64,
squared relative tolerance 1e-12 (relative Frobenius 1e-6).  A step is one
complete adaptive ID of the matrix.  Seeded synthetic data stands in for the
reference's generators throughout.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RBRP matrices/s & ID time at equal rel err, mixed+batched vs plain FP64"
L2_BYTES = 126 * 2**20        # GB300 L2
L2_FLUSH_BYTES = 512 * 2**20  # written between timed steps when an input fits in L2

WORKLOADS = {
    "blocks4096": dict(kind="blocks", nblocks=4096, lo=64, hi=2048, lengthscale=0.5, b=0, tol=1e-8),
    "snn16k": dict(kind="snn", m=16384, n=16384, r=2000, r1=100, amp=10.0, density=0.02, b=64, tol=1e-12),
    "snn8k": dict(kind="snn", m=8192, n=8192, r=2000, r1=100, amp=10.0, density=0.02, b=64, tol=1e-12),
    "snn4k": dict(kind="snn", m=4096, n=4096, r=2000, r1=100, amp=10.0, density=0.02, b=64, tol=1e-12),
    "gexp1000": dict(kind="gexp", m=1000, n=1000, decay=20.0, b=40, tol=1e-12),
    "gmm65k": dict(kind="gmm", m=1024, n=65536, clusters=20, b=32, tol=1e-4),
    "adjoint8k": dict(kind="adjoint", n=8192, dim=8, lengthscale=1.5, b=64, tol=1e-6),
    "idcmp16k": dict(kind="idcmp", d=1000, n=16384, clusters=100, b=32, nb=6, tol=1e-12),
    "cpqr16k": dict(kind="cpqr", d=1000, n=16384, clusters=100, k=192),
}


def describe(name, wl):
    if wl["kind"] == "cpqr":
        return (f"{name}: deterministic CPQR ID (greedy b=1, LAPACK dgeqp3's pivots) to rank {wl['k']} of the C++ "
                f"Gaussian-mixture matrix of gpu/driver.cpp, {wl['d']}x{wl['n']} ({wl['clusters']} clusters), FP64; a step is "
                f"one ID (S, T)")
    if wl["kind"] == "idcmp":
        return (f"{name}: the Gaussian-mixture matrix of gpu/driver.cpp, {wl['d']}x{wl['n']} ({wl['clusters']} clusters, "
                f"point i of cluster c shifted by 10(c+1) in coordinate c), FP64; a step is one RBRP (b={wl['b']}) "
                f"to rank {wl['nb'] * wl['b']}; RandCPQR_OS, RandLUPP_OS and the CPQR ID are timed at the first "
                f"{wl['nb']} RBRP ranks, as gpu/driver.cpp does")
    if wl["kind"] == "adjoint":
        return (f"{name}: fixed-skeleton ID loss ||A - A(:,S) T||^2 + ||T w||^2 and its gradient, Gaussian kernel "
                f"{wl['n']}^2 on N(0, I_{wl['dim']}) points, l={wl['lengthscale']}, S from FP32 RBRP at squared tol "
                f"{wl['tol']:g} (b={wl['b']}); a step is one forward + backward (d/dA and d/dl)")
    if wl["kind"] == "blocks":
        return (f"{name}: {wl['nblocks']} Gaussian-kernel blocks (l={wl['lengthscale']}, 3-D unit-cube clusters "
                f"2-8 apart), m, n log-uniform in [{wl['lo']}, {wl['hi']}], FP32 storage scaled by each block's "
                f"max, squared tol {wl['tol']:g} (rel. Frobenius {np.sqrt(wl['tol']):g}), "
                + ("b autotuned" if wl["b"] <= 0 else f"b={wl['b']}"))
    if wl["kind"] == "gmm":
        return (f"{name}: Gaussian mixture, {wl['n']} points as columns in R^{wl['m']}, {wl['clusters']} clusters "
                f"(weights 2^-c, means N(0, 4I), sigma U[0.1, 1]), FP32 storage, b={wl['b']}, squared tol "
                f"{wl['tol']:g}; every cluster must appear in S")
    if wl["kind"] == "snn":
        return (f"{name}: SNN {wl['m']}x{wl['n']} (2000 rank-one terms, density {wl['density']}), FP32 storage, "
                f"b={wl['b']}, squared tol {wl['tol']:g} (rel. Frobenius {np.sqrt(wl['tol']):g})")
    return (f"{name}: U diag(exp(-i/20)) V^T {wl['m']}x{wl['n']} FP64, b={wl['b']}, "
            f"squared tol {wl['tol']:g}")


def single_input_bytes(wl):
    """Bytes of the matrix a single-matrix workload's timed step reads (FP32 for the mixed form)."""
    return wl["m"] * wl["n"] * (4 if wl["kind"] in ("snn", "gmm") else 8)


def single_config(name, wl):
    """The ``config`` of both arms of a single-matrix workload (identical by construction)."""
    b = single_input_bytes(wl)
    l2 = (f"no flush: the {b / 2**20:.0f} MiB input is larger than L2" if b >= 2 * L2_BYTES
          else f"L2 flushed before every timed step (the {b / 2**20:.0f} MiB input fits)")
    return {"workload": describe(name, wl), "l2": l2}


def make_matrix(wl, seed, torch, device):
    """(A64, A32) column-major CUDA tensors of the workload."""
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    if wl["kind"] == "snn":
        X, w, Y = W.snn_factors(wl["m"], wl["n"], wl["r"], wl["r1"], wl["amp"], wl["density"], seed)
        Xt = torch.from_numpy(X * w).to(device)
        Yt = torch.from_numpy(Y).to(device)
        A64 = (Yt @ Xt.t()).t()           # (m, n) column major
        del Xt, Yt
    elif wl["kind"] == "gmm":
        A, _ = W.gmm(wl["m"], wl["n"], wl["clusters"], seed)
        A64 = torch.from_numpy(A).to(device).t().contiguous().t()
    else:
        A = W.gaussian_exp(wl["m"], wl["n"], decay=wl["decay"], seed=seed)
        A64 = torch.from_numpy(A).to(device).t().contiguous().t()
    A32 = A64.float().t().contiguous().t()
    return A64, A32


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.uuid = uuid
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        cmd = ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.uuid:
            cmd.insert(1, f"--id={self.uuid}")
        try:
            self.proc = subprocess.Popen(cmd, stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except OSError:
            pass
        if self.path and os.path.exists(self.path):
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def model_flops_oracle(o, m, n):
    """Algorithmic flops of an oracle run (same model as the library's phase counters)."""
    f = 2.0 * m * n
    prev = 0
    for blk in o["blocks"]:
        bh, bt = blk["bs_sampled"], blk["bs"]
        nt = n - prev - bt
        f += 2.0 * m * nt * bt + 4.0 * m * prev * bh + 2.0 * m * bh * bh + 4.0 * m * bt * bt
        prev += bt
    return f


def cpu_sample(A64_host, wl, seed, kmax_sample):
    """Time the oracle port on the first blocks of the workload; returns (seconds, flops, desc)."""
    from oracle import rbrp_column_id
    t0 = time.perf_counter()
    o = rbrp_column_id(A64_host, wl["b"], tol=wl["tol"], kmax=kmax_sample, seed=seed)
    dt = time.perf_counter() - t0
    m, n = A64_host.shape
    return dt, model_flops_oracle(o, m, n), o


def threads():
    try:
        from threadpoolctl import threadpool_info
        info = threadpool_info()
        return max([i.get("num_threads", 1) for i in info] or [os.cpu_count()])
    except Exception:
        return os.cpu_count()


def run_reference(args, wl, name):
    """The reference arm: the oracle port of the reference's CPU RBRP on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    kmax_sample = 2 * wl["b"]
    if wl["kind"] == "snn":
        X, w, Y = W.snn_factors(wl["m"], wl["n"], wl["r"], wl["r1"], wl["amp"], wl["density"], 0)
        A = np.asfortranarray((X * w) @ Y.T)
        full_k = min(wl["r"], wl["m"], wl["n"])
    elif wl["kind"] == "gmm":
        A, _ = W.gmm(wl["m"], wl["n"], wl["clusters"], 0)
        full_k = min(wl["m"], wl["n"])
    else:
        A = W.gaussian_exp(wl["m"], wl["n"], decay=wl["decay"], seed=0)
        full_k = None
    times, flops = [], []
    for s in range(args.warmup + args.steps):
        dt, f, o = cpu_sample(A, wl, 0, kmax_sample)
        if s >= args.warmup:
            times.append(dt)
            flops.append(f)
    rate = sum(flops) / sum(times)
    m, n = A.shape
    kf = full_k or o["k"]
    # full-run flop model: average sampled block, k_full ranks, plus the T solve
    nb = max(1, -(-kf // wl["b"]))
    f_full = 2.0 * m * n + sum(2.0 * m * (n - (t + 1) * wl["b"]) * wl["b"] + 4.0 * m * t * wl["b"] * wl["b"]
                               + 6.0 * m * wl["b"] ** 2 for t in range(nb)) + kf * kf * (n - kf)
    value = rate / f_full
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "matrices/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox)",
        "config": single_config(name, wl),
        "cpu_baseline": {"value": value, "unit": "matrices/s", "cores": threads(), "kind": "port",
                         "sample": f"oracle port (numpy/scipy FP64) of the reference's blocked_rpid on the first "
                                   f"{kmax_sample} ranks of the same matrix per step; matrices/s extrapolated by "
                                   f"the algorithmic flop model to k={kf}"},
        "e2e": {"value": value, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


class Ctx:
    """Process / device context shared by the bench legs."""

    def __init__(self, args, device_type="cuda"):
        """One rank: its GPU, NCCL for the timing all-reduce.  ``device_type="cpu"``
        gives the same rank logic over gloo on host tensors (the multi-process tests)."""
        import torch
        import torch.distributed as dist
        self.torch, self.dist = torch, dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        if device_type == "cpu":
            self.device = torch.device("cpu")
            if self.world > 1:
                dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.stream = None
        else:
            torch.cuda.set_device(self.local)
            self.device = torch.device("cuda", self.local)
            if self.world > 1:
                dist.init_process_group("nccl", device_id=self.device)
            self.stream = torch.cuda.current_stream(self.device)
        self.uuid = None
        try:
            self.uuid = "GPU-" + str(torch.cuda.get_device_properties(self.local).uuid)
        except Exception:
            pass
        self.peaks = {}
        try:
            self.peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except OSError:
            pass

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max_over_ranks(self, x):
        t = self.torch.tensor([x], device=self.device, dtype=self.torch.float64)
        if self.world > 1:
            self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def job_rate(self, units_per_rank, ms):
        """Whole-job rate: the units of every rank over the slowest rank's time.
        Returns (units/s, max ms)."""
        ms_max = self.max_over_ranks(ms)
        return self.world * units_per_rank / (ms_max * 1e-3), ms_max

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


def traffic_from_profile(name):
    """DRAM bytes per launch from the committed ncu summary of this workload (or None)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def run_single(args, wl, name, ctx, light=False):
    """One adaptive ID per step of one matrix per rank; returns the JSON line (dict)."""
    torch = ctx.torch
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    seed = ctx.rank
    A64, A32 = make_matrix(wl, seed, torch, ctx.device)
    m, n = A32.shape
    h = Handle(ctx.local)
    stream = ctx.stream
    mixed = wl["kind"] in ("snn", "gmm")
    A = A32 if mixed else A64
    kw = dict(b=wl["b"], tol=wl["tol"], seed=seed)
    warmup, steps = (2, 2) if light else (args.warmup, args.steps)

    for _ in range(warmup):
        r = h.column_id(A, **kw)
    h.set_profiling(True)
    h.reset_phase_stats()
    ctx.barrier()
    torch.cuda.synchronize()
    in_bytes = m * n * A.element_size()
    # inputs that fit in L2 are evicted before every timed step by a write of a larger buffer
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=ctx.device) if in_bytes < 2 * L2_BYTES else None
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(ctx.uuid) as clk:
        if flush is None:
            ev0.record(stream)
            for _ in range(steps):
                r = h.column_id(A, **kw)
            ev1.record(stream)
            torch.cuda.synchronize()
            ms = ev0.elapsed_time(ev1)
        else:
            ms = 0.0
            for _ in range(steps):
                flush.zero_()
                ev0.record(stream)
                r = h.column_id(A, **kw)
                ev1.record(stream)
                torch.cuda.synchronize()
                ms += ev0.elapsed_time(ev1)
    ctx.barrier()
    del flush
    stats = h.phase_stats()
    h.set_profiling(False)
    clocks = clk.summary()
    value, ms_max = ctx.job_rate(steps, ms)

    k = r.k
    rel_err = h.id_error(A)             # squared, on the matrix the ID was computed for
    coverage = None
    if wl["kind"] == "gmm":             # every cluster represented in the skeleton
        from robust_blockwise_random_pivoting_gb300 import workloads as W
        _, labels = W.gmm(wl["m"], wl["n"], wl["clusters"], seed)
        got = len(set(labels[r.perm[:k].cpu().numpy()].tolist()))
        coverage = {"clusters": wl["clusters"], "in_skeleton": got}

    e2e = None
    if not (args.no_e2e or light):
        hostA = torch.empty((n, m), dtype=A.dtype, pin_memory=True).t()
        hostA.copy_(A)
        kcap = min(m, n)
        T_out = torch.empty(kcap * n, dtype=torch.float64, pin_memory=True)
        perm_out = torch.empty(n, dtype=torch.int32, pin_memory=True)
        h.column_id_host(hostA, perm_out=perm_out, T_out=T_out, **kw)
        ctx.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            k_h, _, _, _ = h.column_id_host(hostA, perm_out=perm_out, T_out=T_out, **kw)
        torch.cuda.synchronize()
        dt = ctx.max_over_ranks(time.perf_counter() - t0)
        e2e = {"value": ctx.world * steps / dt, "unit": "matrices/s",
               "h2d_bytes_per_step": int(m * n * A.element_size()),
               "d2h_bytes_per_step": int(4 * n + 8 * k_h * (n - k_h))}
        del hostA, T_out

    plain = None
    if mixed and not args.no_plain:
        hp = Handle(ctx.local)
        hp.column_id(A64, **kw)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rp = hp.column_id(A64, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1)
        plain = {"matrices_per_s": 1e3 / pms, "id_time_ms": pms, "k": rp.k,
                 "rel_err": float(np.sqrt(max(hp.id_error(A64), 0.0)))}
        if coverage is not None:
            plain["clusters_in_skeleton"] = len(set(labels[rp.perm[: rp.k].cpu().numpy()].tolist()))
        hp.close()

    hbm_peak = ctx.peaks.get("hbm_gbs", 6800.0)
    dom = max(("project", "update", "tsolve", "cgs", "panel", "sample", "norms", "finish"),
              key=lambda q: stats[q]["ms"])
    st = stats[dom]
    launches = max(1, st["launches"])
    per_launch_ms = st["ms"] / launches
    achieved = st["bytes"] / launches / (per_launch_ms * 1e-3) / 1e9
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": None,
                "flops_per_s": st["flops"] / (st["ms"] * 1e-3) if st["ms"] else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if ctx.peaks else "fallback 6.8 TB/s"}
    phases = {q: {"ms_per_step": v["ms"] / steps, "launches_per_step": v["launches"] / steps,
                  "GBps": (v["bytes"] / (v["ms"] * 1e-3) / 1e9) if v["ms"] else None,
                  "TFLOPs": (v["flops"] / (v["ms"] * 1e-3) / 1e12) if v["ms"] else None}
              for q, v in stats.items()}
    gpu_launches = int(sum(v["launches"] for v in stats.values()))

    cpu = None
    if ctx.rank == 0 and ctx.world == 1 and not (args.no_cpu or light):
        A_host = A64.cpu().numpy()
        kmax_sample = 2 * wl["b"]
        dt, f, o = cpu_sample(A_host, wl, seed, kmax_sample)
        f_full = sum(v["flops"] for v in stats.values()) / steps
        cpu = {"value": (f / dt) / f_full, "unit": "matrices/s", "cores": threads(), "kind": "port",
               "sample": f"oracle port (numpy/scipy FP64) of the reference's blocked_rpid on the first "
                         f"{kmax_sample} ranks of the same matrix ({dt:.1f} s); matrices/s extrapolated by the "
                         f"algorithmic flop model to the GPU run's trace (k={k}, {r.nblocks} blocks)"}
    h.close()
    del A64, A32
    return {
        "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": ctx.world, "steps": steps,
        "warmup": warmup, "ms_per_step": ms_max / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
        "data": "synthetic (seeded Philox), one independent matrix per rank",
        "config": single_config(name, wl),
        "details": {"precision": "mixed" if mixed else "f64",
                   "k": k, "blocks": r.nblocks, "id_time_ms": ms_max / steps,
                   "rel_err": float(np.sqrt(max(rel_err, 0.0))), "err_est_sq": r.err_est,
                   "plain_f64": plain, "parallelism": f"replicas x{ctx.world}", "cluster_coverage": coverage,
                   "phases": phases},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
        "gpu_launches": gpu_launches,
    }


def block_sample_ids(nblocks, count, seed):
    return np.sort(np.random.default_rng(1000 + seed).choice(nblocks, size=min(count, nblocks), replace=False))


CPU_SAMPLE_BLOCKS = 256   # the seeded block sample both CPU legs time (cpu_baseline and --impl reference)


def batched_cpu_sample(wl, seed, b, count=CPU_SAMPLE_BLOCKS, mats=None, keep=False):
    """The oracle port on a seeded sample of the workload's blocks.

    Each block is one complete ID as the GPU computes it: the adaptive RBRP
    (``blocked_rpid``) and the interpolation matrix T (``interpolation(...,
    mode='sid')``, the oracle's ``interp_sid``).  ``mats`` (FP64 host copies of
    the sampled blocks) replaces the host-side generation; with ``keep`` the
    oracle runs are returned for the parity check.  Returns ``(seconds, count,
    description, ids, mats, runs)``."""
    from oracle import interp_sid, rbrp_column_id
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    ids = block_sample_ids(wl["nblocks"], count, seed)
    if mats is None:
        shapes = W.kernel_block_shapes(wl["nblocks"], wl["lo"], wl["hi"], seed)
        mats = [W.kernel_block_scaled(int(shapes[q][0]), int(shapes[q][1]), q, wl["lengthscale"], seed)
                .astype(np.float64) for q in ids]
    runs = []
    t0 = time.perf_counter()
    for q, A in zip(ids, mats):
        o = rbrp_column_id(A, b, tol=wl["tol"], seed=seed * wl["nblocks"] + int(q))
        if 0 < o["k"] < A.shape[1]:
            interp_sid(A, o["perm"], o["k"])
        if keep:
            runs.append(o)
    dt = time.perf_counter() - t0
    return dt, len(ids), (f"oracle port (numpy/scipy FP64) of the reference's blocked_rpid plus interpolation "
                          f"(mode='sid') for T, on a seeded sample of {len(ids)} of the {wl['nblocks']} blocks "
                          f"(same shape distribution, same sample in both CPU legs), b={b}; "
                          f"matrices/s = sample size / time"), ids, mats, runs


def batched_config(name, wl):
    """The ``config`` of both arms of a batched workload (identical by construction)."""
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    sh = W.kernel_block_shapes(wl["nblocks"], wl["lo"], wl["hi"], 0)
    gb = float((sh[:, 0] * sh[:, 1]).sum()) * 4 / 1e9
    l2 = (f"no flush: the {gb:.1f} GB of inputs are larger than L2" if gb > 0.2 else
          f"the {gb:.2f} GB of inputs may sit in L2 (a profiling subset)")
    return {"workload": describe(name, wl), "l2": l2}


def same_rank_parity(wl, seed, b, ids, mats, runs, res, rel):
    """The GPU's IDs of the sampled blocks against the oracle's at the same rank.

    For block q of rank k, the oracle's squared error at rank k comes from its
    adaptive run with the same Philox key (``oracle.error_at_rank``: its
    skeleton at the block boundary k, or - when k falls inside one of its
    sampled panels, where a robust-filter decision near its threshold kept one
    pivot more or fewer - that panel's first pivots); the ratio is un-squared
    (relative Frobenius), GPU / oracle.  Blocks whose rank and ordered skeleton
    equal the oracle's follow its trajectory; the others are listed."""
    from oracle import error_at_rank
    ratios, same, diverged = [], [], []
    for j, (q, A) in enumerate(zip(ids, mats)):
        k = int(res.k[q])
        perm = res.perms[q].cpu().numpy()
        o = runs[j]
        e_ref, how = error_at_rank(A, k, b, tol=wl["tol"], seed=seed * wl["nblocks"] + int(q), run=o)
        e_gpu = float(rel[q]) ** 2
        r = float(np.sqrt(max(e_gpu, 1e-24) / max(e_ref, 1e-24)))
        ratios.append(r)
        if k == o["k"] and bool(np.array_equal(perm[:k], o["perm"][:k])):
            same.append(r)
        else:
            first = int(np.argmax(perm[:min(k, o["k"])] != o["perm"][:min(k, o["k"])])) if min(k, o["k"]) else 0
            diverged.append({"block": int(q), "k": k, "k_oracle": int(o["k"]), "first_differing_position": first,
                             "oracle_last_block_start": int(o["blocks"][-1]["i"]), "ratio": r, "how": how})
    r = np.array(ratios)
    return {"blocks": len(ids), "max_err_ratio_same_rank": float(r.max()),
            "median_err_ratio_same_rank": float(np.median(r)),
            "blocks_on_oracle_trajectory": len(same),
            "max_err_ratio_on_oracle_trajectory": float(max(same)) if same else None,
            "diverged": diverged,
            "definition": "relative Frobenius ID error of the GPU's S and T over the oracle's (FP64, same FP32 "
                          "values, same Philox key) at the GPU's rank; 'on oracle trajectory' = same rank and "
                          "ordered skeleton"}


def tight_tolerance_leg(args, wl, ctx, As, seed, b, t_cap, tol=1e-12, subset=64):
    """The throughput target's tolerance: squared 1e-12 (relative Frobenius 1e-6).

    The batched form over all blocks (own plan, CUDA-event timed launches) and
    the plain FP64 one-launch-per-matrix form on a seeded subset of the same
    blocks, each with its largest relative error checked in FP64 on the device."""
    torch = ctx.torch
    from robust_blockwise_random_pivoting_gb300.rbrp import Batch, Handle
    nb = len(As)
    h = Handle(ctx.local)
    bt = Batch(h, As, b=b, tol=tol, seed=seed * nb, t_rank_cap=t_cap)
    bt.run()
    bt.results()
    steps = max(1, min(args.steps, 5))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(ctx.stream)
    for _ in range(steps):
        bt.run(ctx.stream)
    ev1.record(ctx.stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    res = bt.results()

    def rel_err(A, perm, k, T):
        n = A.shape[1]
        if k == 0 or k == n:
            return 0.0 if k == n else 1.0
        p = perm.long()
        A64 = A.double()
        return float(torch.linalg.norm(A64[:, p[k:]] - A64[:, p[:k]] @ T) / torch.linalg.norm(A64))
    rel = [rel_err(A, res.perms[q], int(res.k[q]), res.Ts[q]) if res.status[q] == 0 else float("nan")
           for q, A in enumerate(As)]
    batched = {"matrices_per_s": nb / (ms * 1e-3), "ms_per_launch": ms, "launches_timed": steps,
               "k_mean": float(res.k.mean()), "k_max": int(res.k.max()), "status_ok": int((res.status == 0).sum()),
               "rel_err_max": float(np.nanmax(rel))}
    h.close()
    ids = block_sample_ids(nb, subset, seed)
    hs = Handle(ctx.local)
    sub = [As[q].double().t().contiguous().t() for q in ids]
    hs.column_id(sub[0], b=b, tol=tol, seed=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ks = []
    for q, A in zip(ids, sub):
        ks.append(hs.column_id(A, b=b, tol=tol, seed=seed * nb + int(q)).k)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    errs = []
    for q, A in zip(ids, sub):
        hs.column_id(A, b=b, tol=tol, seed=seed * nb + int(q))
        errs.append(float(np.sqrt(max(hs.id_error(A), 0.0))))
    hs.close()
    plain = {"subset": len(ids), "matrices_per_s": len(ids) / dt, "ms_per_matrix": 1e3 * dt / len(ids),
             "k_mean": float(np.mean(ks)), "rel_err_max": float(np.max(errs))}
    return {"tol_squared": tol, "rel_frobenius": float(np.sqrt(tol)), "b": b, "batched_mixed": batched,
            "plain_f64_one_launch_per_matrix": plain,
            "speedup_batched_vs_plain_f64": batched["matrices_per_s"] / plain["matrices_per_s"]}


def run_batched(args, wl, name, ctx):
    """All blocks of the workload in one persistent launch per step; returns the JSON line (dict)."""
    torch = ctx.torch
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    from robust_blockwise_random_pivoting_gb300.rbrp import Batch, Handle
    seed = ctx.rank
    nb = wl["nblocks"]
    blocks = W.kernel_blocks_device(nb, wl["lo"], wl["hi"], wl["lengthscale"], seed, ctx.device)
    shapes = [tuple(A.shape) for A in blocks]
    # all blocks packed in one device buffer (column major each, 16-byte aligned starts),
    # also the layout of the e2e host buffer
    from robust_blockwise_random_pivoting_gb300.rbrp import packed_offsets
    offs, sizes = packed_offsets(shapes)
    pack = torch.zeros(int(offs[-1]), dtype=torch.float32, device=ctx.device)
    As = []
    for q, ((m, n), A) in enumerate(zip(shapes, blocks)):
        v = pack[int(offs[q]): int(offs[q]) + int(sizes[q])].view(n, m).t()
        v.copy_(A)
        As.append(v)
    del blocks
    h = Handle(ctx.local)
    t_cap = 64
    t_plan = time.perf_counter()
    bt = Batch(h, As, b=wl["b"], tol=wl["tol"], seed=seed * nb, t_rank_cap=t_cap)
    t_plan = time.perf_counter() - t_plan
    info = bt.info()
    stream = ctx.stream
    for _ in range(args.warmup):
        bt.run()
        res = bt.results()
    ctx.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(ctx.uuid) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            bt.run(stream)
        ev1.record(stream)
        torch.cuda.synchronize()
    ctx.barrier()
    ms = ev0.elapsed_time(ev1)
    clocks = clk.summary()
    res = bt.results()
    value, ms_max = ctx.job_rate(args.steps * nb, ms)
    ms_launch = ms / args.steps

    # quality: relative Frobenius error of every ID against the block in FP64 (device GEMMs)
    rel = np.zeros(nb)
    for q, A in enumerate(As):
        k = int(res.k[q])
        m, n = shapes[q]
        if k == 0 or k == n or res.Ts[q] is None:
            rel[q] = 0.0 if k == n else (1.0 if k == 0 else np.nan)
            continue
        p = res.perms[q].long()
        A64 = A.double()
        E = A64[:, p[k:]] - A64[:, p[:k]] @ res.Ts[q]
        rel[q] = float(torch.linalg.norm(E) / torch.linalg.norm(A64))
    ok = int((res.status == 0).sum())

    # one profiled launch: in-kernel phase cycle shares
    bt.set_profiling(True)
    bt.run()
    bt.results()
    cyc = bt.phase_cycles()
    bt.set_profiling(False)
    tot = sum(cyc.values()) or 1.0
    phases = {q: round(v / tot, 4) for q, v in cyc.items()}

    alg_bytes = float(res.alg_bytes.sum())
    alg_flops = float(res.alg_flops.sum())
    hbm_peak = ctx.peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (ms_launch * 1e-3) / 1e9
    roofline = {"kernel": "k_rbrp_batched", "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": traffic_from_profile("k_rbrp_batched_blocks4096.md"),
                "alg_bytes_per_launch": alg_bytes, "flops_per_s": alg_flops / (ms_launch * 1e-3),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if ctx.peaks else "fallback 6.8 TB/s"}

    # one launch per matrix: plain FP64 and FP32 mixed, on a seeded subset of the same blocks
    single = None
    if not args.no_plain:
        ids = block_sample_ids(nb, 64, seed)
        hs = Handle(ctx.local)
        single = {"subset": len(ids), "b": info["b"]}
        for label, dt in (("plain_f64", torch.float64), ("f32_one_launch", torch.float32)):
            sub = [As[q].to(dt).t().contiguous().t() for q in ids]
            kw = dict(b=info["b"], tol=wl["tol"])
            hs.column_id(sub[0], seed=0, **kw)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            errs, ks = [], []
            for j, (q, A) in enumerate(zip(ids, sub)):
                r = hs.column_id(A, seed=seed * nb + int(q), **kw)
                ks.append(r.k)
            torch.cuda.synchronize()
            dt_s = time.perf_counter() - t0
            for A, q in zip(sub, ids):
                r = hs.column_id(A, seed=seed * nb + int(q), **kw)
                errs.append(float(np.sqrt(max(hs.id_error(A), 0.0))))
            single[label] = {"matrices_per_s": len(ids) / dt_s, "ms_per_matrix": 1e3 * dt_s / len(ids),
                             "k_mean": float(np.mean(ks)), "rel_err_max": float(np.max(errs))}
            del sub
        single["batched_same_subset"] = {"k_mean": float(res.k[ids].mean()), "rel_err_max": float(rel[ids].max())}
        hs.close()

    # end to end: pinned host blocks in, one H2D copy, the graph launch, perms + T + results out
    e2e = None
    if not args.no_e2e:
        host = torch.empty(pack.numel(), dtype=torch.float32, pin_memory=True)
        host.copy_(pack)
        perm_h = torch.empty(bt.perm_buf.numel(), dtype=torch.int32, pin_memory=True)
        T_h = torch.empty(bt.T_buf.numel(), dtype=torch.float64, pin_memory=True)

        seg = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

        def step():
            seg[0].record()
            pack.copy_(host, non_blocking=True)
            seg[1].record()
            bt.run()
            seg[2].record()
            perm_h.copy_(bt.perm_buf, non_blocking=True)
            T_h.copy_(bt.T_buf, non_blocking=True)
            seg[3].record()
            return bt.results()
        step()
        ctx.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        split = np.zeros(3)
        for _ in range(args.steps):
            step()
            split += [seg[i].elapsed_time(seg[i + 1]) for i in range(3)]
        torch.cuda.synchronize()
        dt = ctx.max_over_ranks(time.perf_counter() - t0)
        split /= args.steps
        sequential = {"value": ctx.world * args.steps * nb / dt, "unit": "matrices/s",
                      "ms_h2d": float(split[0]), "ms_run": float(split[1]), "ms_d2h": float(split[2]),
                      "h2d_GBps": float(pack.numel() * 4 / split[0] / 1e6)}
        del perm_h, T_h
        # the pipelined host API: groups of problems, copies overlapped with the IDs on two streams
        from robust_blockwise_random_pivoting_gb300.rbrp import HostBatch
        hb = HostBatch(host, shapes, parts=2, b=info["b"], tol=wl["tol"], seed=seed * nb, t_rank_cap=t_cap,
                       device=ctx.local)

        def hstep():
            hb.run()
            return hb.results()
        hstep()
        ctx.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            hstep()
        torch.cuda.synchronize()
        dt = ctx.max_over_ranks(time.perf_counter() - t0)
        pipelined = {"value": ctx.world * args.steps * nb / dt, "unit": "matrices/s",
                     "api": f"rbrp.HostBatch, {len(hb.groups)} groups: copies on one stream overlapped with "
                            f"the groups' launches on another"}
        hb.close()
        sequential.update({"h2d_bytes_per_step": int(pack.numel() * 4), "d2h_bytes_per_step": int(hb.d2h_bytes + nb * 56),
                           "api": "one pinned H2D copy of the packed blocks, rbrp.Batch.run (one graph launch), "
                                  "perm and T copied to pinned host buffers, Batch.results()"})
        # host-resident form: rbrp.Batch over views of the pinned pack; the kernel reads each
        # block once over the host link (its norms pass stages it in the CTA's workspace) and
        # writes perm and T to pinned host memory, so the transfers overlap the other CTAs' IDs
        hviews = [host[int(offs[q]): int(offs[q]) + int(sizes[q])].view(n, m).t() for q, (m, n) in enumerate(shapes)]
        hz_handle = Handle(ctx.local)
        hz = Batch(hz_handle, hviews, b=info["b"], tol=wl["tol"], seed=seed * nb, t_rank_cap=t_cap)

        def zstep():
            hz.run()
            return hz.results()
        for _ in range(max(1, args.warmup)):
            zres = zstep()
        same = bool(np.array_equal(zres.k, res.k) and np.array_equal(zres.err_est, res.err_est))
        ctx.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            zres = zstep()
        torch.cuda.synchronize()
        dt = ctx.max_over_ranks(time.perf_counter() - t0)
        t_bytes = int(sum(int(k) * (n - int(k)) * 8 for k, (_, n) in zip(zres.k, shapes) if 0 < int(k) < n))
        host_resident = {
            "value": ctx.world * args.steps * nb / dt, "unit": "matrices/s", "ms_step": 1e3 * dt / args.steps,
            "h2d_bytes_per_step": int(pack.numel() * 4),
            "d2h_bytes_per_step": int(hz.perm_buf.numel() * 4 + t_bytes + nb * 56),
            "results_equal_device_batch": same,
            "api": "rbrp.Batch over views of the pinned host pack (one graph launch; the kernel reads each "
                   "block in place once and writes perm and T to pinned host memory), Batch.results()"}
        del hz, hviews
        hz_handle.close()
        # headline: the host-resident form, declared in advance; the other host-buffer forms beside it
        e2e = dict(host_resident)
        e2e["form"] = "host_resident"
        # the host link's own rate on this machine (the sequential form's pinned H2D copy of the same
        # bytes): the time the inputs alone need, against the step
        link = float(sequential["h2d_GBps"])
        ms_inputs = pack.numel() * 4 / (link * 1e6)
        e2e["host_link"] = {"GBps": link, "ms_for_inputs": ms_inputs,
                            "frac_of_step": ms_inputs / host_resident["ms_step"],
                            "note": ("pinned H2D rate of one cudaMemcpyAsync of the same inputs in this run; the "
                                     "host-resident kernel reads them in place at about this rate, so "
                                     "frac_of_step near 1 means the link bounds the step")}
        e2e["other_forms"] = {"sequential": sequential, "pipelined": pipelined}
        del host

    cpu = parity = None
    if ctx.rank == 0 and ctx.world == 1 and not args.no_cpu:
        # the oracle on the GPU's own FP32 values of the sampled blocks: timed as the CPU
        # baseline, then (outside the timing) the checker of the same-rank parity
        ids = block_sample_ids(nb, CPU_SAMPLE_BLOCKS, seed)
        mats = [As[q].double().cpu().numpy() for q in ids]
        dt, cnt, desc, ids, mats, runs = batched_cpu_sample(wl, seed, info["b"], mats=mats, keep=True)
        cpu = {"value": cnt / dt, "unit": "matrices/s", "cores": threads(), "kind": "port", "sample": desc}
        parity = same_rank_parity(wl, seed, info["b"], ids, mats, runs, res, rel)
        del mats, runs

    tight = None
    if not args.no_plain:
        tight = tight_tolerance_leg(args, wl, ctx, As, seed, info["b"], 256)

    single_matrix = None
    if not args.no_single and ctx.world == 1:
        sl = run_single(args, WORKLOADS["snn16k"], "snn16k", ctx, light=True)
        single_matrix = {"workload": sl["config"]["workload"], "id_time_ms": sl["details"]["id_time_ms"],
                         "k": sl["details"]["k"], "rel_err": sl["details"]["rel_err"],
                         "plain_f64": sl["details"]["plain_f64"], "roofline": sl["roofline"],
                         "clocks": sl["clocks"], "timing": "2 warm-up + 2 timed IDs"}
    h.close()
    return {
        "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": ctx.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded Philox points), one independent batch per rank",
        "config": batched_config(name, wl),
        "parity": parity, "tol_1e-12": tight,
        "details": {"precision": "mixed", "problems": nb,
                   "elements": int(offs[-1]), "b": info["b"], "ctas": info["ctas"],
                   "ctas_per_sm": info["ctas_per_sm"], "plan_s": t_plan, "autotune_ms": info["ms_autotune"],
                   "k_mean": float(res.k.mean()), "k_max": int(res.k.max()), "blocks_mean": float(res.nblocks.mean()),
                   "status_ok": ok, "rel_err_max": float(np.nanmax(rel)), "rel_err_mean": float(np.nanmean(rel)),
                   "one_launch_per_matrix": single, "single_matrix_snn16k": single_matrix,
                   "parallelism": f"replicas x{ctx.world}", "launch": "one CUDA graph (queue reset + kernel)",
                   "phase_cycle_share": phases},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
        "gpu_launches": args.steps,
    }


def run_adjoint(args, wl, name, ctx):
    """Forward + backward of the differentiable fixed-skeleton ID per step; returns the JSON line (dict)."""
    torch = ctx.torch
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id_loss, gaussian_kernel_matrix
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    seed = ctx.rank
    n = wl["n"]
    P = torch.from_numpy(W.gaussian_kernel_points(n, wl["dim"], seed)).to(ctx.device)
    h = Handle(ctx.local)
    A0 = gaussian_kernel_matrix(P, wl["lengthscale"]).float().t().contiguous().t()
    t0 = time.perf_counter()
    r = h.column_id(A0, b=wl["b"], tol=wl["tol"], seed=seed)
    torch.cuda.synchronize()
    t_rbrp = time.perf_counter() - t0
    S = r.perm[: r.k].clone()
    k = r.k
    w = torch.randn(n, generator=torch.Generator(device="cpu").manual_seed(7 + seed)).to(ctx.device)

    def step():
        ls = torch.tensor(wl["lengthscale"], dtype=torch.float64, device=ctx.device, requires_grad=True)
        A = gaussian_kernel_matrix(P, ls).float()
        loss = fixed_skeleton_id_loss(A, S, w, b=wl["b"], handle=h)
        loss.backward()
        return loss, ls.grad
    for _ in range(args.warmup):
        loss, gl = step()
    ctx.barrier()
    torch.cuda.synchronize()
    with ClockSampler(ctx.uuid) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            loss, gl = step()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    clocks = clk.summary()
    dt = ctx.max_over_ranks(dt)
    value = ctx.world * args.steps / dt

    # the adjoint kernels alone (CUDA events): forward fixed ID + loss, then fixed ID + gradient
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_loss_and_grad
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(ctx.stream)
    fixed_skeleton_loss_and_grad(h, A0, S, w, wl["b"], grad=False)
    ev[1].record(ctx.stream)
    _, G = fixed_skeleton_loss_and_grad(h, A0, S, w, wl["b"], grad=True)
    ev[2].record(ctx.stream)
    torch.cuda.synchronize()
    ms_fwd, ms_bwd = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    nc = n - k
    gemm_flops = 2.0 * (2.0 * n * nc * k)   # E = B - C T and E T^T

    # FP64 reference gradient (torch autograd through a QR least-squares T) on the same FP32 matrix
    check = None
    if not args.no_plain:
        A64 = A0.double().requires_grad_(True)
        mask = torch.ones(n, dtype=torch.bool, device=ctx.device)
        mask[S.long()] = False
        rd = torch.nonzero(mask).flatten()
        C, B = A64[:, S.long()], A64[:, rd]
        Q, R = torch.linalg.qr(C)
        T = torch.linalg.solve_triangular(R, Q.t() @ B, upper=True)
        E = B - C @ T
        lref = (E * E).sum() + ((T @ w.double()[rd]) ** 2).sum()
        lref.backward()
        check = {"loss": float(loss.item()), "loss_fp64": float(lref.item()),
                 "grad_A_rel_err": float((torch.linalg.norm(G.double() - A64.grad) / torch.linalg.norm(A64.grad)).item()),
                 "grad_l": float(gl.item())}
        del A64, C, B, Q, R, T, E
    # the adjoint call alone (its forward factorisation done just before, outside the timing):
    # both tcgen05 GEMMs and the small kernels around them
    import ctypes
    from robust_blockwise_random_pivoting_gb300.adjoint import fixed_skeleton_id
    fixed_skeleton_id(h, A0, S, wl["b"])
    Gbuf = torch.empty((n, n), dtype=torch.float32, device=ctx.device).t()
    wf = w.float().contiguous()
    lossv = ctypes.c_double()
    t_adj = []
    for _ in range(3):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e[0].record(ctx.stream)
        rc = h.lib.rbrp_fixed_id_adjoint_f32(h.h, n, n, ctypes.c_void_p(A0.data_ptr()), n,
                                             ctypes.c_void_p(wf.data_ptr()), ctypes.c_float(1.0),
                                             ctypes.c_void_p(Gbuf.data_ptr()), n, ctypes.byref(lossv))
        e[1].record(ctx.stream)
        torch.cuda.synchronize()
        if rc != 0:
            raise RuntimeError(f"adjoint call failed ({rc})")
        t_adj.append(e[0].elapsed_time(e[1]))
    ms_adj = min(t_adj)
    del Gbuf
    # 3xTF32 ceiling in useful FLOP/s: TF32 issues at half the dense BF16 rate (1.1 of 2.25
    # PFLOP/s nominal) and each product takes 3 MMAs; BF16 from the measured peaks
    bf16 = ctx.peaks.get("bf16_tflops", 1900.0)
    ceil_3xtf32 = bf16 * (1.1 / 2.25) / 3.0
    achieved = gemm_flops / (ms_adj * 1e-3) / 1e12
    h.close()
    return {
        "metric": METRIC, "value": value, "unit": "forward+backward/s", "n_gpus": ctx.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Philox points)",
        "config": {"workload": describe(name, wl), "k": k, "rbrp_forward_s": t_rbrp, "ms_fixed_id_and_loss": ms_fwd,
                   "ms_fixed_id_and_gradient": ms_bwd, "check": check},
        "roofline": {"kernel": "k_gemm_tc<EpiE> + k_gemm_tc<EpiG> (tcgen05 3xTF32)", "bound": "tensor",
                     "achieved": achieved, "peak": ceil_3xtf32, "unit": "TFLOP/s", "frac": achieved / ceil_3xtf32,
                     "traffic": None, "ms_adjoint_call": ms_adj,
                     "peak_source": ("MEASURED_PEAKS.json bf16_tflops (measured) x 1.1/2.25 (TF32 / BF16 nominal) / 3 "
                                     "(3 MMAs per product); useful GEMM flops 2 x 2 m (n-k) k over the whole "
                                     "adjoint call (both GEMMs, the z solve and the small kernels)"
                                     if ctx.peaks else "fallback 1.9 PFLOP/s BF16 x 1.1/2.25 / 3")},
        "cpu_baseline": None, "e2e": None, "clocks": clocks, "gpu_launches": None,
    }


def run_idcmp(args, wl, name, ctx):
    """The comparison of gpu/driver.cpp: RBRP, then the comparison IDs at RBRP's first ranks; returns the JSON line."""
    torch = ctx.torch
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    from robust_blockwise_random_pivoting_gb300.sketch_ids import cpqr_id, rand_cpqr_os, rand_lupp_os
    seed = ctx.rank
    A_host = W.driver_gmm(wl["n"], wl["d"], wl["clusters"], seed)
    A = torch.from_numpy(A_host).to(ctx.device).t().contiguous().t()
    h = Handle(ctx.local)
    nrm2 = float((A * A).sum())
    kmax = wl["nb"] * wl["b"]
    kw = dict(b=wl["b"], tol=wl["tol"], kmax=kmax, seed=seed)

    def sq_err(sk, rd, T):
        E = A[:, rd.long()] - A[:, sk.long()] @ T
        return float((E * E).sum()) / nrm2

    for _ in range(args.warmup):
        r = h.column_id(A, **kw)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ctx.barrier()
    torch.cuda.synchronize()
    with ClockSampler(ctx.uuid) as clk:
        ev[0].record(ctx.stream)
        for _ in range(args.steps):
            r = h.column_id(A, **kw)
        ev[1].record(ctx.stream)
        torch.cuda.synchronize()
    clocks = clk.summary()
    dt = ctx.max_over_ranks(ev[0].elapsed_time(ev[1]) * 1e-3)
    ranks = [int(x) for x in r.ranks[: wl["nb"]]]
    rbrp_err = [float(x) for x in r.residuals[: wl["nb"]]]

    def timed(fn, k):
        fn(k)                                   # warm: workspaces and one-time attributes
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        e[0].record(ctx.stream)
        sk, rd, T = fn(k)
        e[1].record(ctx.stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]), sq_err(sk, rd, T)

    methods = {
        "RandCPQR_OS": lambda k: rand_cpqr_os(A, k, seed=seed, handle=h),
        "RandLUPP_OS": lambda k: rand_lupp_os(A, k, seed=seed, handle=h),
        "CPQR_ID": lambda k: cpqr_id(A, k, handle=h),
    }
    comparison = {"ranks": ranks, "RBRP": {"sq_rel_err": rbrp_err, "ms_to_last_rank": 1e3 * dt / args.steps}}
    for label, fn in methods.items():
        res = [timed(fn, k) for k in ranks]
        comparison[label] = {"ms": [x[0] for x in res], "sq_rel_err": [x[1] for x in res]}
    cpu = None
    if not args.no_cpu and ctx.rank == 0:
        dtc, f, o = cpu_sample(A_host, wl, seed, 2 * wl["b"])
        cpu = {"value": 1.0 / dtc, "unit": "samples/s", "cores": threads(), "kind": "port",
               "sample": f"oracle port (numpy/scipy FP64) of blocked_rpid on the first {2 * wl['b']} ranks "
                         f"of the same matrix, {dtc:.3f} s"}
    h.close()
    return {
        "metric": METRIC, "value": ctx.world * args.steps / dt, "unit": "matrices/s", "n_gpus": ctx.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Philox)",
        "config": {"workload": describe(name, wl), "comparison": comparison},
        "cpu_baseline": cpu, "e2e": None, "clocks": clocks, "gpu_launches": None,
    }


def run_cpqr(args, wl, name, ctx):
    """The deterministic CPQR ID (the CPQR baseline of gpu/driver.cpp) per step; returns the JSON line."""
    torch = ctx.torch
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    from robust_blockwise_random_pivoting_gb300.sketch_ids import cpqr_id
    seed = ctx.rank
    A_host = W.driver_gmm(wl["n"], wl["d"], wl["clusters"], seed)
    A = torch.from_numpy(A_host).to(ctx.device).t().contiguous().t()
    m, n = A.shape
    h = Handle(ctx.local)
    for _ in range(args.warmup):
        sk, rd, T = cpqr_id(A, wl["k"], handle=h)
    h.set_profiling(True)
    h.reset_phase_stats()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ctx.barrier()
    torch.cuda.synchronize()
    with ClockSampler(ctx.uuid) as clk:
        ev[0].record(ctx.stream)
        for _ in range(args.steps):
            sk, rd, T = cpqr_id(A, wl["k"], handle=h)
        ev[1].record(ctx.stream)
        torch.cuda.synchronize()
    clocks = clk.summary()
    stats = h.phase_stats()
    h.set_profiling(False)
    dt = ctx.max_over_ranks(ev[0].elapsed_time(ev[1]) * 1e-3)
    E = A[:, rd.long()] - A[:, sk.long()] @ T
    rel_err = float(torch.linalg.norm(E) / torch.linalg.norm(A))
    st = stats["project"]
    launches = max(1, st["launches"])
    per_launch_s = st["ms"] * 1e-3 / launches
    hbm_peak = ctx.peaks.get("hbm_gbs", 6800.0)
    achieved = st["bytes"] / launches / per_launch_s / 1e9
    cpu = None
    if not args.no_cpu and ctx.rank == 0:
        from oracle import rbrp_column_id
        ks = 16
        t0 = time.perf_counter()
        rbrp_column_id(A_host, 1, tol=None, kmax=ks, seed=seed, mode="gp")
        dtc = time.perf_counter() - t0
        cpu = {"value": 1.0 / (dtc * wl["k"] / ks), "unit": "matrices/s", "cores": threads(), "kind": "port",
               "sample": f"oracle port (numpy/scipy FP64) in greedy mode, b=1, first {ks} ranks of the same "
                         f"matrix ({dtc:.2f} s), scaled to rank {wl['k']} by the rank count"}
    h.close()
    return {
        "metric": METRIC, "value": ctx.world * args.steps / dt, "unit": "matrices/s", "n_gpus": ctx.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Philox)",
        "config": {"workload": describe(name, wl), "k": int(sk.numel()), "rel_err": rel_err,
                   "l2": f"no flush: the {m * n * 8 / 2**20:.0f} MiB input is larger than L2",
                   "phases": {q: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps}
                              for q, v in stats.items()}},
        "roofline": {"kernel": "k_project_skinny<double, 1>", "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                     "limiter": "the FP64 pipe (one FMA per element of A; GB300's FP64 rate)",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if ctx.peaks else "fallback 6.8 TB/s"},
        "cpu_baseline": cpu, "e2e": None, "clocks": clocks,
        "gpu_launches": int(sum(v["launches"] for v in stats.values())),
    }


def run_reference_batched(args, wl, name):
    """Reference arm for the batched workload: the oracle port on the host cores.

    The timed steps split the seeded 256-block sample of ``cpu_baseline`` between
    them (step s takes its s-th share), so K steps time the whole sample once and
    the run stays within seconds; each warm-up step runs the sample's first 4
    blocks.  ``value`` = sampled blocks / the timed steps' total time."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import interp_sid, rbrp_column_id
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    b = 16
    ids = block_sample_ids(wl["nblocks"], CPU_SAMPLE_BLOCKS, 0)
    shapes = W.kernel_block_shapes(wl["nblocks"], wl["lo"], wl["hi"], 0)
    mats = [W.kernel_block_scaled(int(shapes[q][0]), int(shapes[q][1]), q, wl["lengthscale"], 0).astype(np.float64)
            for q in ids]

    def one(j):
        o = rbrp_column_id(mats[j], b, tol=wl["tol"], seed=int(ids[j]))
        if 0 < o["k"] < mats[j].shape[1]:
            interp_sid(mats[j], o["perm"], o["k"])
    for _ in range(args.warmup):
        for j in range(min(4, len(ids))):
            one(j)
    times, counts = [], []
    for part in np.array_split(np.arange(len(ids)), max(1, args.steps)):
        t0 = time.perf_counter()
        for j in part:
            one(int(j))
        times.append(time.perf_counter() - t0)
        counts.append(len(part))
    value = sum(counts) / sum(times)
    desc = (f"oracle port (numpy/scipy FP64) of the reference's blocked_rpid plus interpolation (mode='sid') for "
            f"T, on a seeded sample of {len(ids)} of the {wl['nblocks']} blocks (the cpu_baseline sample), b={b}, "
            f"split over the {max(1, args.steps)} timed steps; matrices/s = sample size / total time")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Philox points)", "config": batched_config(name, wl),
        "cpu_baseline": {"value": value, "unit": "matrices/s", "cores": threads(), "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="blocks4096", choices=sorted(WORKLOADS))
    ap.add_argument("--no-plain", action="store_true", help="skip the one-launch-per-matrix comparisons")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-single", action="store_true", help="skip the snn16k single-matrix figure")
    ap.add_argument("--nblocks", type=int, default=0,
                    help="batched workloads: a smaller problem count of the same shape distribution (profiling)")
    ap.add_argument("--hi", type=int, default=0, help="batched workloads: a smaller largest m and n (profiling)")
    ap.add_argument("--b", type=int, default=0, help="batched workloads: fixed block size instead of the autotuner")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload])
    if wl["kind"] == "blocks":
        if args.nblocks > 0:
            wl["nblocks"] = args.nblocks
        if args.hi > 0:
            wl["hi"] = max(wl["lo"], args.hi)
        if args.b > 0:
            wl["b"] = args.b
    if args.impl == "reference":
        if wl["kind"] == "adjoint":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no differentiable ID"}))
            return
        if wl["kind"] in ("idcmp", "cpqr"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference's comparison IDs are "
                              "cuSOLVER/MAGMA GPU code; its CPU RBRP is the reference arm of the other workloads"}))
            return
        if wl["kind"] == "blocks":
            run_reference_batched(args, wl, args.workload)
        else:
            run_reference(args, wl, args.workload)
        return
    ctx = Ctx(args)
    if wl["kind"] == "blocks":
        line = run_batched(args, wl, args.workload, ctx)
    elif wl["kind"] == "adjoint":
        line = run_adjoint(args, wl, args.workload, ctx)
    elif wl["kind"] == "idcmp":
        line = run_idcmp(args, wl, args.workload, ctx)
    elif wl["kind"] == "cpqr":
        line = run_cpqr(args, wl, args.workload, ctx)
    else:
        line = run_single(args, wl, args.workload, ctx)
    if ctx.rank == 0:
        print(json.dumps(line))
    ctx.close()


if __name__ == "__main__":
    main()
