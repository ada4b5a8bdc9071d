#!/usr/bin/env python
"""Benchmark of the GB300 VNEC mxv (SpMV) path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One step = one y = A x over the whole synthetic matrix.  Default workload:
the 2^24-row R-MAT power-law matrix (2^28 generated edges, a=.57 b=c=.19,
duplicates merged, values U(0,1), x U(-1,1), seed 1) in plain FP64 — the
configuration the headline metric is quoted on.  The matrix and x are
resident in HBM before timing; the L2 is flushed (a 512 MiB device write)
before every timed step, and each step is bracketed by CUDA events on the
launching stream.  `value` is algorithmic bytes / time (GB/s):
    B = nnz*(8 + 4) + (n_rows + 1)*4 + n_cols*8 + n_rows*8
(values + int32 columns, row offsets, x once, y once).

Extra keys: `roofline` (dominant kernel's live event time vs the measured HBM
copy peak), `e2e` (the same metric through the C-ABI host entry point with
pinned host x and y, copies inside the timed region), `cpu_baseline` (the
oracle's restatement of the reference's VNEC-L FP64 on this host's cores,
reference protocol 1 warm-up + up to 40 calls), `clocks` (nvidia-smi sampled
during the timed region), `rel_error` (against the compensated FP64 oracle).

Multi-GPU: the path does not partition across GPUs in this build, so N GPUs
run N independent replicas of the workload (scaling "weak").

`--impl reference` times the reference's own CPU algorithm for the path on
the host cores (the oracle restatement; the reference's AVX-512 build cannot
run on an aarch64 host) and prints the same line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpMV GB/s (% of GB300 HBM peak), mixed/batched vs plain FP64 at fixed rel. error"
L2_FLUSH_BYTES = 512 << 20


def workload(name: str):
    from vnec_gb300 import generators as G

    if name == "rmat24":
        m = G.rmat(24, 1 << 28, 0.57, 0.19, 0.19, seed=1)
        x = G.vector(m.n_cols, lo=-1.0, hi=1.0, seed=1)
        desc = "rmat_scale24_edges2^28_a.57_b.19_c.19_dedup_fp64"
    elif name == "uniform64k":
        m = G.uniform_k(65536, 16, seed=0)
        x = G.vector(m.n_cols, seed=0)
        desc = "uniform_n65536_k16_fp64"
    elif name == "rmat22":
        m = G.rmat(22, 1 << 26, 0.57, 0.19, 0.19, seed=1)
        x = G.vector(m.n_cols, lo=-1.0, hi=1.0, seed=1)
        desc = "rmat_scale22_edges2^26_a.57_b.19_c.19_dedup_fp64"
    elif name == "stencil256":
        m = G.stencil27(256, seed=0)
        x = G.vector(m.n_cols, seed=0)
        desc = "stencil27_256^3_fp64"
    else:
        raise SystemExit(f"unknown workload {name}")
    return m, x, desc


def algorithmic_bytes(m) -> int:
    off = 8 if (m.n_rows + m.nnz) >= (1 << 31) - 1 else 4
    return m.nnz * 12 + (m.n_rows + 1) * off + m.n_cols * 8 + m.n_rows * 8


def measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)"
    except Exception:
        return 6800.0, "fallback (6.8 TB/s)"


def profiled_traffic(kernel: str, wl: str):
    """dram bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{wl}.md")
    try:
        for line in open(p):
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1].strip()))
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi samples (200 ms) filtered to a wall-clock window."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(index)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self, t0: float, t1: float):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = []
        for line in self.f.read().splitlines():
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                ts = time.mktime(time.strptime(parts[0].split(".")[0], "%Y/%m/%d %H:%M:%S"))
                ts += float("0." + parts[0].split(".")[1]) if "." in parts[0] else 0.0
                rows.append((ts, float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        inside = [r for r in rows if t0 - 0.25 <= r[0] <= t1 + 0.25] or rows
        if not inside:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[1] for r in inside])), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": reasons, "samples": len(inside)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reference_cores_and_parts() -> tuple[int, int, str]:
    arch = platform.machine()
    # NUM_THREADS of the reference build for this host (SpB_mxv.h:19,27).
    nparts = 48 if arch in ("aarch64", "arm64") else 36
    return os.cpu_count() or 1, nparts, arch


def cpu_time_L(m, x, warm: int, reps: int, budget_s: float) -> tuple[float, int, str]:
    """Seconds per call of the reference's VNEC-L FP64 on the host (oracle port)."""
    from oracle import oracle as O

    cores, nparts, arch = reference_cores_and_parts()
    t1 = O.time_L_f64(m, x, nparts, warm=warm, reps=1)
    reps = int(max(1, min(reps, budget_s / max(t1, 1e-9))))
    secs = O.time_L_f64(m, x, nparts, warm=0, reps=reps)
    return secs, reps, f"VNEC-L FP64 restated (oracle port), {nparts} OpenMP partitions/threads on {cores} {arch} cores"


def run_reference(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    m, x, desc = workload(args.workload)
    B = algorithmic_bytes(m)
    cores, nparts, arch = reference_cores_and_parts()
    from oracle import oracle as O

    per_call = O.time_L_f64(m, x, nparts, warm=args.warmup, reps=args.steps)
    value = B / per_call / 1e9
    sample = (f"full workload, {args.warmup} warm-up + {args.steps} timed SpMV_VNEC_L_FP64 calls (the reference "
              f"dispatch for n >= 3e6), restated in C (oracle port); {nparts} OpenMP threads on {cores} {arch} cores")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(per_call * 1e3, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": desc, "n_rows": m.n_rows, "nnz": m.nnz, "algorithmic_bytes": B},
            "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import torch

    from vnec_gb300 import api

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    t_gen = time.time()
    m, xv, desc = workload(args.workload)
    t_gen = time.time() - t_gen
    B = algorithmic_bytes(m)
    t_plan = time.time()
    kernel = {"L": api.KERNEL_L, "S": api.KERNEL_S}[args.kernel]
    plan = api.Plan(m, kernel=kernel)
    t_plan = time.time() - t_plan
    info = plan.info()
    stream = torch.cuda.Stream(device=dev)
    x = torch.from_numpy(xv).to(dev)
    y = torch.empty(m.n_rows, dtype=torch.float64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    sampler = ClockSampler(dev.index)
    plan.set_profiling(True)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1)
            plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
    stream.synchronize()

    # ---- device-timed steps -------------------------------------------------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    main_ms = []
    barrier()
    torch.cuda.synchronize()
    w0 = time.time()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(k)
            starts[k].record(stream)
            plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
            ends[k].record(stream)
            main_ms.append(plan.kernel_ms()[0])
    torch.cuda.synchronize()
    barrier()
    w1 = time.time()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = float(np.sum(step_ms))
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = B * args.steps * ws / (total_ms / 1e3) / 1e9
    y_dev = y.cpu().numpy()

    # ---- end to end through the C ABI with pinned host buffers --------------
    plan.set_profiling(False)
    hx = torch.from_numpy(xv).pin_memory()
    hy = torch.empty(m.n_rows, dtype=torch.float64).pin_memory()
    hx_np, hy_np = hx.numpy(), hy.numpy()
    for _ in range(max(1, args.warmup)):
        plan.mxv_host(hx_np, hy_np)
    e2e_s = 0.0
    e2e_steps = max(1, args.steps // 4)
    barrier()
    for _ in range(e2e_steps):
        flush.fill_(3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plan.mxv_host(hx_np, hy_np)
        e2e_s += time.perf_counter() - t0
    barrier()
    w2 = time.time()
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    clocks = sampler.stop(w0, w2)
    e2e_value = B * e2e_steps * ws / e2e_s / 1e9
    if not np.array_equal(hy_np, y_dev):
        raise RuntimeError("host-path and device-path results differ")

    # ---- accuracy against the compensated FP64 oracle ------------------------
    from oracle import oracle as O

    y_ref, cond = O.spmv_neumaier(m, xv)
    rel = O.rowwise_error(y_dev, y_ref, cond)

    peak, peak_src = measured_peaks()
    kname = {"L": "mp2_kernel", "S": "sliced_kernel"}[args.kernel]
    achieved = B / (np.mean(main_ms) / 1e3) / 1e9
    traffic = profiled_traffic(kname, args.workload)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, resident in HBM before timing)",
        "config": {"workload": desc, "n_rows": m.n_rows, "n_cols": m.n_cols, "nnz": m.nnz,
                   "algorithmic_bytes": B,
                   "kernel": {"L": "merge-path CSR (VNEC-L counterpart)",
                              "S": "sliced row groups (VNEC-S counterpart)"}[args.kernel],
                   "arithmetic": "fp64 fma" if info.arithmetic != 2 else "df32 (double-float on FP32 pipe)",
                   "tile": f"{info.threads_per_block}x{info.items_per_thread}", "tiles": info.num_tiles,
                   "l2": "flushed before every timed step (512 MiB device write, outside the events)",
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "gen_s": round(t_gen, 2), "plan_build_s": round(t_plan, 2)},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_src,
                     "traffic": traffic, "mean_kernel_ms": round(float(np.mean(main_ms)), 5),
                     "fixup_share": round(1.0 - float(np.sum(main_ms)) / total_ms, 4)},
        "e2e": {"value": round(e2e_value, 3), "unit": "GB/s", "h2d_bytes_per_step": m.n_cols * 8,
                "d2h_bytes_per_step": m.n_rows * 8, "steps": e2e_steps,
                "path": "SpB_mxv_host_ext (pinned host x/y; H2D x, SpMV, D2H y per call)"},
        "gpu_launches": args.steps * info.launches_per_call,
        "clocks": clocks,
        "rel_error": {"max_rowwise": float(rel.max()), "median_rowwise": float(np.median(rel)),
                      "criterion": "|y-yhat| <= 1e-12 * sum|a x| (compensated FP64 oracle)"},
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        secs, reps, sample = cpu_time_L(m, xv, warm=1, reps=40, budget_s=args.cpu_budget)
        cores, _, _ = reference_cores_and_parts()
        line["cpu_baseline"] = {"value": round(B / secs / 1e9, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                                "sample": f"full workload, 1 warm-up + {reps} calls; {sample}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.free()
    if ws > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="rmat24", choices=["rmat24", "rmat22", "uniform64k", "stencil256"])
    ap.add_argument("--kernel", default="S", choices=["L", "S"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU-baseline timing")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
