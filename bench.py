#!/usr/bin/env python
"""Benchmark of the GB300 adaptive RBRP column ID (one JSON line on stdout).

Workload (default ``snn16k``): the sparse non-negative low-rank-plus-tail
matrix A = sum_{j<=100} (10/j) x_j y_j^T + sum_{100<j<=2000} (1/j) x_j y_j^T,
16384 x 16384, x_j, y_j i.i.d. with density 0.02 and Uniform[0,1] nonzeros,
stored dense FP32 (FP64 copy for the plain form and the error check);
b = 64, squared relative tolerance 1e-12 (relative Frobenius 1e-6), Philox
seed = rank.  Seeded synthetic data stands in for the reference's generators.

A step is one complete adaptive ID of the matrix (norms, sampling, panels,
projections, stop, T = R11^{-1} R12), so ``value`` is matrices/s.  The matrix
(1 GiB) is larger than L2, so no flush is needed between steps.
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

WORKLOADS = {
    "snn16k": dict(kind="snn", m=16384, n=16384, r=2000, r1=100, amp=10.0, density=0.02, b=64, tol=1e-12),
    "snn8k": dict(kind="snn", m=8192, n=8192, r=2000, r1=100, amp=10.0, density=0.02, b=64, tol=1e-12),
    "snn4k": dict(kind="snn", m=4096, n=4096, r=2000, r1=100, amp=10.0, density=0.02, b=64, tol=1e-12),
    "gexp1000": dict(kind="gexp", m=1000, n=1000, decay=20.0, b=40, tol=1e-12),
}


def describe(name, wl):
    if wl["kind"] == "snn":
        return (f"{name}: SNN {wl['m']}x{wl['n']} (2000 rank-one terms, density {wl['density']}), FP32 storage, "
                f"b={wl['b']}, squared tol {wl['tol']:g} (rel. Frobenius {np.sqrt(wl['tol']):g})")
    return (f"{name}: U diag(exp(-i/20)) V^T {wl['m']}x{wl['n']} FP64, b={wl['b']}, "
            f"squared tol {wl['tol']:g}")


def make_matrix(wl, seed, torch, device):
    """(A64, A32) column-major CUDA tensors of the workload."""
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    if wl["kind"] == "snn":
        X, w, Y = W.snn_factors(wl["m"], wl["n"], wl["r"], wl["r1"], wl["amp"], wl["density"], seed)
        Xt = torch.from_numpy(X * w).to(device)
        Yt = torch.from_numpy(Y).to(device)
        A64 = (Yt @ Xt.t()).t()           # (m, n) column major
        del Xt, Yt
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
        "config": {"workload": describe(name, wl)},
        "cpu_baseline": {"value": value, "unit": "matrices/s", "cores": threads(), "kind": "port",
                         "sample": f"oracle port (numpy/scipy FP64) of the reference's blocked_rpid on the first "
                                   f"{kmax_sample} ranks of the same matrix per step; matrices/s extrapolated by "
                                   f"the algorithmic flop model to k={kf}"},
        "e2e": {"value": value, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="snn16k", choices=sorted(WORKLOADS))
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl, args.workload)
        return

    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=device)

    def barrier():
        if world > 1:
            dist.barrier()

    from robust_blockwise_random_pivoting_gb300.rbrp import Handle
    seed = rank
    A64, A32 = make_matrix(wl, seed, torch, device)
    m, n = A32.shape
    h = Handle(local)
    stream = torch.cuda.current_stream(device)
    mixed = wl["kind"] == "snn"
    A = A32 if mixed else A64
    kw = dict(b=wl["b"], tol=wl["tol"], seed=seed)

    for _ in range(args.warmup):
        r = h.column_id(A, **kw)
    h.set_profiling(True)
    h.reset_phase_stats()
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        pass
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(uuid) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            r = h.column_id(A, **kw)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    stats = h.phase_stats()
    h.set_profiling(False)
    clocks = clk.summary()
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * args.steps / (ms_max * 1e-3)

    # quality of the last timed result, against the FP64 matrix
    k = r.k
    rel_err = h.id_error(A)             # squared, on the matrix the ID was computed for
    perm = r.perm.clone()
    T = r.T

    # end to end through the host-buffer entry point (pinned host A, perm and T out)
    e2e = None
    if not args.no_e2e:
        hostA = torch.empty((n, m), dtype=A.dtype, pin_memory=True).t()
        hostA.copy_(A)
        kcap = min(m, n)
        T_out = torch.empty(kcap * n, dtype=torch.float64, pin_memory=True)
        perm_out = torch.empty(n, dtype=torch.int32, pin_memory=True)
        for _ in range(1):
            h.column_id_host(hostA, perm_out=perm_out, T_out=T_out, **kw)
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            k_h, _, _, _ = h.column_id_host(hostA, perm_out=perm_out, T_out=T_out, **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        tt = torch.tensor([dt], device=device, dtype=torch.float64)
        if world > 1:
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        dt = float(tt.item())
        e2e = {"value": world * args.steps / dt, "unit": "matrices/s",
               "h2d_bytes_per_step": int(m * n * A.element_size()),
               "d2h_bytes_per_step": int(4 * n + 8 * k_h * (n - k_h))}
        del hostA, T_out

    # plain FP64 single-launch form on the same matrix (the comparison the metric names)
    plain = None
    if mixed and not args.no_plain:
        hp = Handle(local)
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
        hp.close()

    # dominant phase and its roofline (algorithmic bytes over measured launch time)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    dom = max(("project", "update", "tsolve", "cgs", "panel", "sample", "norms", "finish"),
              key=lambda q: stats[q]["ms"])
    st = stats[dom]
    launches = max(1, st["launches"])
    per_launch_ms = st["ms"] / launches
    achieved = st["bytes"] / launches / (per_launch_ms * 1e-3) / 1e9
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": None,
                "flops_per_s": st["flops"] / (st["ms"] * 1e-3) if st["ms"] else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s"}
    phases = {q: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps,
                  "GBps": (v["bytes"] / (v["ms"] * 1e-3) / 1e9) if v["ms"] else None,
                  "TFLOPs": (v["flops"] / (v["ms"] * 1e-3) / 1e12) if v["ms"] else None}
              for q, v in stats.items()}
    gpu_launches = int(sum(v["launches"] for v in stats.values()))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        A_host = A64.cpu().numpy()
        kmax_sample = 2 * wl["b"]
        dt, f, o = cpu_sample(A_host, wl, seed, kmax_sample)
        f_full = sum(v["flops"] for v in stats.values()) / args.steps
        cpu = {"value": (f / dt) / f_full, "unit": "matrices/s", "cores": threads(), "kind": "port",
               "sample": f"oracle port (numpy/scipy FP64) of the reference's blocked_rpid on the first "
                         f"{kmax_sample} ranks of the same matrix ({dt:.1f} s); matrices/s extrapolated by the "
                         f"algorithmic flop model to the GPU run's trace (k={k}, {r.nblocks} blocks)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
            "data": "synthetic (seeded Philox), one independent matrix per rank",
            "config": {"workload": describe(args.workload, wl), "precision": "mixed" if mixed else "f64",
                       "k": k, "blocks": r.nblocks, "id_time_ms": ms_max / args.steps,
                       "rel_err": float(np.sqrt(max(rel_err, 0.0))), "err_est_sq": r.err_est,
                       "plain_f64": plain, "parallelism": f"replicas x{world}",
                       "l2": "no flush: the 1 GiB input is larger than L2", "phases": phases},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": gpu_launches,
        }
        print(json.dumps(line))
    h.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
