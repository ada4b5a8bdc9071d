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
copy peak), `e2e` (the same metric through the C-ABI host entry points with
page-locked host x and y, every step's x copy in and y copy out inside the
timed region: `value` from pipelined calls, SpB_mxv_host_async_ext, where
consecutive steps overlap their copies with the neighbouring SpMVs;
`sync_value` from one blocking SpB_mxv_host_ext call per step), `cpu_baseline` (the
oracle's restatement of the reference's VNEC-L FP64 on this host's cores,
reference protocol 1 warm-up + up to 40 calls), `clocks` (nvidia-smi sampled
during the timed region), `rel_error` (against the compensated FP64 oracle),
`legs` (per matrix — the headline matrix and, for R-MAT 2^24, the 256^3
27-point stencil — the plain FP64 sliced kernel, its FP32 / BF16+row-scale /
FP32 hi+lo forms, the learned and rule-based kernel selections and the learned
selection of the FP32 form (the mixed-precision, learned-tuned plan): median ms
over --leg-steps flushed calls, speed-up over plain FP64, row-wise error),
`batch_legs` (the batched form on 512 uneven matrices, k = 1 and 32, FP64 /
FP32 / DF32, autotuned, 5 graph-replayed steps each).

`--workload batch512` measures the batched multi-right-hand-side form instead
(512 uneven matrices, k = 1..32, one graph-replayed persistent launch per step).

Multi-GPU: one matrix is not partitioned across GPUs, so N GPUs run N
independent replicas of the workload (scaling "weak").

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
# --precision: sliced-kernel form of the main plan (api.PREC_*), its dtype label and error bound.
PRECISIONS = {"fp64": 0, "fp32": 1, "bf16": 2, "df32": 3}
PREC_DTYPE = {"fp64": "f64", "fp32": "f32 (fp64 reductions)", "bf16": "bf16 x row scale (fp32 products, fp64 reductions)",
              "df32": "f32 hi+lo (double-float)"}
PREC_TOL = {"fp64": 1e-12, "fp32": 1e-6, "bf16": 1e-2, "df32": 1e-12}
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
    elif name in ("stencil256", "stencil128"):
        g = int(name[len("stencil"):])
        m = G.stencil27(g, seed=0)
        x = G.vector(m.n_cols, seed=0)
        desc = f"stencil27_{g}^3_fp64"
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


def replica_max(value: float, device=None) -> float:
    """Max of `value` over the ranks of the default process group (the value
    itself when no group is initialised); device: where the collective's
    tensor lives (the rank's GPU for NCCL, the CPU for gloo)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(bytes_per_step: int, steps: int, world: int, max_ms: float) -> float:
    """Whole-job GB/s of `world` replicas that each ran `steps` steps, timed by
    the slowest rank (weak scaling: every replica does the full workload)."""
    return bytes_per_step * steps * world / (max_ms / 1e3) / 1e9


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


def cpu_time_L(m, x, warm: int, reps: int, budget_s: float) -> tuple[float, int, str, str]:
    """Seconds per call of the reference harness's dispatch on the host cores
    (VNEC-L FP64 for n >= 3e6 rows, else IRD_VNEC's D or S; test_spmv_vnec.cpp:
    197-256), the timed calls, a description and the kind: "reference" when the
    reference library built from its own sources for this host is present
    (oracle/_ref; on the aarch64 GPU host its ARM_NEON build), else "port"
    (the oracle's restatement with the reference's compile-time constants)."""
    from oracle import oracle as O

    cores, nparts, arch = reference_cores_and_parts()
    if O.ref_available():
        b = O.ref_build()
        t1, _ = O.ref_time_f64(m, x, 0, warm, 1)
        reps = int(max(1, min(reps, budget_s / max(t1, 1e-9))))
        secs, name = O.ref_time_f64(m, x, 0, 0, reps)
        flavour = "ARM_NEON" if b is O.ARM else "X86_SIMD (AVX-512)"
        return secs, reps, (f"{name} FP64 of the reference itself (its {flavour} build, compiled from its own "
                            f"sources, NUM_THREADS {b['nparts']}) on {cores} {arch} cores"), "reference"
    build = dict(O.ARM if arch in ("aarch64", "arm64") else O.X86, nparts=nparts)
    if m.n_rows >= 3_000_000:
        name = "VNEC-L"

        def run(w, r):
            return O.time_L_f64(m, x, nparts, warm=w, reps=r)
    else:
        name = f"VNEC-S (IRD {O.ird(m, build=build)[1]:.3f})"

        def run(w, r):
            return O.time_S_f64(m, x, build=build, warm=w, reps=r)
    t1 = run(warm, 1)
    reps = int(max(1, min(reps, budget_s / max(t1, 1e-9))))
    secs = run(0, reps)
    return (secs, reps, f"{name} FP64 restated (oracle port), {nparts} OpenMP partitions/threads on {cores} {arch} "
                        "cores", "port")


def time_plan_device(plan, x, y, flush, stream, steps: int, warmup: int) -> list[float]:
    """CUDA-event times (ms) of `steps` device-path calls, L2 flushed before each."""
    import torch

    with torch.cuda.stream(stream):
        for _ in range(warmup):
            plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i, (a, b) in enumerate(ev):
            flush.fill_(i)
            a.record(stream)
            plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
            b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def pipelined_e2e(plan, hx_np, ny: int, steps: int):
    """`steps` independent host-vector calls through SpB_mxv_host_async_ext
    (page-locked x and y; every call copies x in, runs the SpMV and copies y
    out, consecutive calls overlapping on three streams), timed on the wall
    clock from the first enqueue to SpB_VNEC_host_wait_ext.  Returns the
    seconds and the y of the last call."""
    import torch

    hys = [torch.empty(ny, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    for i in range(2):  # warm-up: allocates both buffer slots
        plan.mxv_host_async(hx_np, hys[i])
    plan.host_wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        plan.mxv_host_async(hx_np, hys[i % 2])
    plan.host_wait()
    return time.perf_counter() - t0, hys[(steps - 1) % 2]


def form_legs(m, xv, B: int, flush, stream, steps: int, warmup: int) -> dict:
    """Plain FP64 and the precision forms of the sliced kernel on one matrix, plus
    the learned kernel selection: median ms, throughput in the plain form's
    algorithmic bytes (so ratios are time ratios), speed-up over plain FP64 and
    row-wise error against the compensated FP64 oracle."""
    import torch

    from oracle import oracle as O
    from vnec_gb300 import api

    y_ref, cond = O.spmv_neumaier(m, xv)
    x = torch.from_numpy(xv).to(flush.device)
    y = torch.empty(m.n_rows, dtype=torch.float64, device=flush.device)
    legs = {}
    S = dict(kernel=api.KERNEL_S, items_per_thread=-1)  # unroll timed on the matrix at plan build
    forms = [("fp64", S), ("fp32", dict(S, precision=api.PREC_FP32)),
             ("bf16_rowscale", dict(S, precision=api.PREC_BF16)),
             ("df32_hilo", dict(S, precision=api.PREC_DF32)),
             ("learned", dict(kernel=api.KERNEL_LEARNED)), ("rule", dict(kernel=api.KERNEL_RULE)),
             ("learned_fp32", dict(kernel=api.KERNEL_LEARNED, precision=api.PREC_FP32))]
    base = None
    for name, kw in forms:
        t0 = time.time()
        plan = api.Plan(m, **kw)
        build_s = time.time() - t0
        ms = float(np.median(time_plan_device(plan, x, y, flush, stream, steps, warmup)))
        rel = O.rowwise_error(y.cpu().numpy(), y_ref, cond)
        leg = {"ms": round(ms, 5), "gbs_plain_bytes": round(B / ms / 1e6, 1), "launches": plan.info().launches_per_call,
               "unroll": plan.info().items_per_thread,
               "max_rel_error": float(rel.max()), "median_rel_error": float(np.median(rel)),
               "plan_build_s": round(build_s, 2)}
        if name in ("learned", "rule", "learned_fp32"):
            cfg, how = api.plan_choice(plan)
            leg["config"] = api.tune_configs()[cfg]
            leg["how"] = ["direct", "learned", "search", "rule", "fallback-search"][how]
        if base is None:
            base = ms
        leg["speedup_vs_fp64"] = round(base / ms, 3)
        legs[name] = leg
        plan.free()
    # The reference API's own call sequence for matrices of >= 3e6 rows
    # (test_spmv_vnec.cpp:197,235-256): Build_VNEC_L, then SpMV_VNEC_L_FP64.
    if m.n_rows >= 3_000_000:
        t0 = time.time()
        A = api.Matrix.from_csr(m)
        h = api.Build_VNEC_L(A)
        build_s = time.time() - t0

        class _Handle:
            def mxv_device(self, d_x, d_y, s):
                api._check(api.lib().SpB_mxv_device_ext(h, d_x, d_y, s or None) == api.SpB_SUCCESS, "mxv")

        try:
            ms = float(np.median(time_plan_device(_Handle(), x, y, flush, stream, steps, warmup)))
            rel = O.rowwise_error(y.cpu().numpy(), y_ref, cond)
            legs["build_vnec_l"] = {"ms": round(ms, 5), "gbs_plain_bytes": round(B / ms / 1e6, 1),
                                    "max_rel_error": float(rel.max()), "plan_build_s": round(build_s, 2),
                                    "speedup_vs_fp64": round(base / ms, 3),
                                    "path": "Build_VNEC_L + SpMV_VNEC_L_FP64 handle (reference API flow)"}
        finally:
            api.VNEC_L_free(h)
            del A
    return legs


def gather_ceiling_leg(m, x, flush, stream, spmv_ms: float, steps: int = 10) -> dict:
    """The device's ceiling for a kernel that gathers x once per nonzero: the
    measurement kernel (SpB_VNEC_stream_gather_ext: per item a coalesced
    value and column read, one gather of x, one FP64 FMA, no row structure)
    on this matrix's own column stream in CSR order and on uniform random
    columns over windows of x of 1 MB, 16.8 MB and all of x; items per second
    beside the SpMV kernel's nonzeros per second."""
    import torch

    from vnec_gb300 import api

    dev = x.device
    n = m.nnz
    val = torch.from_numpy(np.ascontiguousarray(m.val[:n], dtype=np.float64)).to(dev)
    out = torch.empty(api.STREAM_GATHER_BLOCKS, dtype=torch.float64, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)
    res = {}
    for name, w in (("matrix_csr_order", m.n_cols), ("uniform_window_1MB", 1 << 17),
                    ("uniform_window_16.8MB", 1 << 21), ("uniform_all_of_x", m.n_cols)):
        if name == "matrix_csr_order":
            col = torch.from_numpy(np.ascontiguousarray(m.col[:n], dtype=np.int32)).to(dev)
        else:
            col = torch.randint(0, w, (n,), generator=gen, device=dev, dtype=torch.int32)
        with torch.cuda.stream(stream):
            for _ in range(3):
                api.stream_gather(x.data_ptr(), m.n_cols, col.data_ptr(), val.data_ptr(), n, out.data_ptr(),
                                  stream.cuda_stream)
            ts = []
            for i in range(steps):
                flush.fill_(i)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                api.stream_gather(x.data_ptr(), m.n_cols, col.data_ptr(), val.data_ptr(), n, out.data_ptr(),
                                  stream.cuda_stream)
                b.record(stream)
                b.synchronize()
                ts.append(a.elapsed_time(b))
        ms = float(np.median(ts))
        res[name] = {"ms": round(ms, 5), "g_items_per_s": round(n / ms / 1e6, 1),
                     "gbs_stream_and_window": round((12.0 * n + 8.0 * w) / ms / 1e6, 1)}
        del col
    res["spmv_kernel_g_nnz_per_s"] = round(n / spmv_ms / 1e6, 1)
    res["spmv_vs_csr_order_ceiling"] = round(res["matrix_csr_order"]["ms"] / spmv_ms, 3)
    res["how"] = ("SpB_VNEC_stream_gather_ext on the same nonzero count, L2 flushed before each call; the "
                  "SpMV kernel also writes y and reads its task and row metadata")
    return res


# Held-out records of the tuner's data set (never trained on): seeds 2000-2199
# and the large records with (seed - 3000) % 4 == 3.
TUNER_LIVE_SEEDS = (2003, 2026, 2049, 2072, 2095, 2118, 2141, 2164, 2187, 3003, 3007)


def tuner_live_leg(seeds=TUNER_LIVE_SEEDS, reps: int = 3) -> dict:
    """Regret of the learned selection measured live on this GPU: for held-out
    matrices of the tuner's generator mix, the configuration the built-in model
    picks against a fresh exhaustive autotune of every configuration."""
    from vnec_gb300 import api
    from vnec_gb300.tuner import dataset

    rows, regrets, b_learned, b_best, t_learned, t_best = [], [], 0, 0, 0.0, 0.0
    t0 = time.time()
    for sd in seeds:
        m, fam, desc = dataset.sample(sd)
        choice, _, ood = api.learned_choice(m)
        ms, best = api.autotune(m, reps=reps)
        ok = np.isfinite(ms)
        chosen_ms = float(ms[choice]) if ok[choice] else float("inf")
        best_ms = float(np.min(ms[ok]))
        r = chosen_ms / best_ms - 1.0
        regrets.append(r)
        bytes_ = dataset.algorithmic_bytes(m)
        b_learned += bytes_
        t_learned += chosen_ms
        t_best += best_ms
        rows.append({"seed": sd, "matrix": desc, "n_rows": m.n_rows, "nnz": m.nnz, "learned": int(choice),
                     "best": int(best), "ms_learned": round(chosen_ms, 4), "ms_best": round(best_ms, 4),
                     "regret": round(r, 4), "out_of_range": ood})
        m.free()
    return {"matrices": rows, "mean_regret": round(float(np.mean(regrets)), 4),
            "max_regret": round(float(np.max(regrets)), 4),
            "aggregate_gbs_learned": round(b_learned / t_learned / 1e6, 1),
            "aggregate_gbs_exhaustive": round(b_learned / t_best / 1e6, 1),
            "seconds": round(time.time() - t0, 1),
            "how": f"exhaustive autotune ({reps} timed calls per configuration) on this GPU vs the model's choice"}


def run_reference(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    # Inputs come from the oracle's own build of the seeded generators (same
    # source, same matrices): this arm maps no library of the product.
    from oracle import oracle as O
    from vnec_gb300 import generators as G

    if not os.path.exists(O.GEN_SO):
        O.build()
    G.use_library(O.GEN_SO)
    if args.workload == "batch512":
        from vnec_gb300 import generators as G

        mats = G.batch_lognormal(args.batch_mats, seed=0)
        k = int(args.rhs.split(",")[-1])
        cb = batch_cpu_baseline(mats, k, args.cpu_budget)
        B = batch_bytes(sum(m.nnz for m in mats), sum(m.n_rows for m in mats), sum(m.n_cols for m in mats),
                        len(mats), k)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "GB/s", "n_gpus": ws,
                "steps": 1, "warmup": 1, "ms_per_step": round(B / (cb["value"] * 1e9) * 1e3, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded generator)",
                "config": {"workload": f"batch512_lognormal_fp64_k{k}", "desc": BATCH_DESC, "algorithmic_bytes": B},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    m, x, desc = workload(args.workload)
    B = algorithmic_bytes(m)
    cores, _, _ = reference_cores_and_parts()
    per_call, reps, how, kind = cpu_time_L(m, x, warm=args.warmup, reps=args.steps,
                                           budget_s=max(args.cpu_budget, 60.0))
    value = B / per_call / 1e9
    sample = (f"full workload, {args.warmup} warm-up + {reps} timed calls of the reference harness's dispatch "
              f"(L for n >= 3e6, else IRD's choice): {how}")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(per_call * 1e3, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": desc, "n_rows": m.n_rows, "nnz": m.nnz, "algorithmic_bytes": B},
            "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": kind,
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
    kernel = {"L": api.KERNEL_L, "S": api.KERNEL_S, "D": api.KERNEL_D}[args.kernel]
    # Sliced plans time their unroll (4/8/12/16 loads in flight) on the matrix at build.
    prec = PRECISIONS[args.precision]
    if prec != api.PREC_FP64 and args.kernel != "S":
        raise SystemExit("--precision applies to the sliced kernel (--kernel S)")
    plan = api.Plan(m, kernel=kernel, items_per_thread=args.unroll if args.kernel == "S" else 0, precision=prec,
                    shared_patterns=0 if args.shared_patterns == "on" else -1)
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
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1)
            plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
    stream.synchronize()

    # ---- device-timed steps (nothing but the calls between the events) -------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    w0 = time.time()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            if args.l2 == "flushed":
                flush.fill_(k)
            starts[k].record(stream)
            plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
            ends[k].record(stream)
    torch.cuda.synchronize()
    barrier()
    w1 = time.time()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = replica_max(float(np.sum(step_ms)), dev)
    value = replica_throughput(B, args.steps, ws, total_ms)
    y_dev = y.cpu().numpy()

    # ---- main kernel's own duration (roofline): a separate pass in which the
    # plan records events around each of its launches ------------------------
    main_ms, call_ms = [], []
    plan.set_profiling(True)
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            if args.l2 == "flushed":
                flush.fill_(k)
            c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            c0.record(stream)
            plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
            c1.record(stream)
            main_ms.append(plan.kernel_ms()[0])
            c1.synchronize()
            call_ms.append(c0.elapsed_time(c1))
    plan.set_profiling(False)
    torch.cuda.synchronize()

    # ---- end to end through the C ABI with pinned host buffers --------------
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
    pipe_steps = max(20, args.steps)
    pipe_s, hy_pipe = pipelined_e2e(plan, hx_np, m.n_rows, pipe_steps)
    barrier()
    w2 = time.time()
    e2e_s = replica_max(e2e_s, dev)
    pipe_s = replica_max(pipe_s, dev)
    clocks = sampler.stop(w0, w2)
    e2e_value = replica_throughput(B, e2e_steps, ws, e2e_s * 1e3)
    pipe_value = replica_throughput(B, pipe_steps, ws, pipe_s * 1e3)
    if not np.array_equal(hy_np, y_dev) or not np.array_equal(hy_pipe, y_dev):
        raise RuntimeError("host-path and device-path results differ")

    # ---- accuracy against the compensated FP64 oracle ------------------------
    from oracle import oracle as O

    y_ref, cond = O.spmv_neumaier(m, xv)
    rel = O.rowwise_error(y_dev, y_ref, cond)

    peak, peak_src = measured_peaks()
    kname = {"L": "mp2_kernel" if info.pipeline_stages else "mp_spmv_kernel", "D": "dense_block_kernel",
             "S": "sliced_kernel" if prec == api.PREC_FP64 else "sliced_mixed_kernel"}[args.kernel]
    # The kernel's own algorithmic bytes: stored value size of the form, 2-byte
    # columns (plus a first column per row) where 16-bit deltas are used.
    B_form = info.algorithmic_bytes if args.kernel in ("S", "D") else B
    achieved = B_form / (np.mean(main_ms) / 1e3) / 1e9
    traffic = profiled_traffic(kname, args.workload + ("" if prec == api.PREC_FP64 else "_" + args.precision) +
                               ("_noshared" if prec != api.PREC_FP64 and args.shared_patterns == "off" else ""))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": PREC_DTYPE[args.precision],
        "data": "synthetic (seeded generator, resident in HBM before timing)",
        "config": {"workload": desc + ("" if prec == api.PREC_FP64 else f"_{args.precision}_form"),
                   "n_rows": m.n_rows, "n_cols": m.n_cols, "nnz": m.nnz,
                   "algorithmic_bytes": B, "form_bytes": B_form,
                   "shared_patterns": args.shared_patterns if prec != api.PREC_FP64 else "n/a",
                   "value_bytes": "plain FP64 bytes (value and e2e are time ratios across forms)",
                   "kernel": {"L": "merge-path CSR (VNEC-L counterpart)",
                              "S": "sliced row groups (VNEC-S counterpart)",
                              "D": "dense blocks of 4 columns (VNEC-D counterpart)"}[args.kernel],
                   "arithmetic": "fp64 fma" if info.arithmetic != 2 else "df32 (double-float on FP32 pipe)",
                   "tile": f"{info.threads_per_block}x{info.items_per_thread}", "tiles": info.num_tiles,
                   "l2": ("flushed before every timed step (512 MiB device write, outside the events)"
                          if args.l2 == "flushed" else "warm: no flush between steps (inputs may stay in L2)"),
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "gen_s": round(t_gen, 2), "plan_build_s": round(t_plan, 2)},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_src,
                     "traffic": traffic, "mean_kernel_ms": round(float(np.mean(main_ms)), 5),
                     "fixup_share": round(max(0.0, 1.0 - float(np.sum(main_ms)) / float(np.sum(call_ms))), 4)},
        "e2e": {"value": round(pipe_value, 3), "unit": "GB/s", "h2d_bytes_per_step": m.n_cols * 8,
                "d2h_bytes_per_step": m.n_rows * 8, "steps": pipe_steps,
                "path": "SpB_mxv_host_async_ext: independent calls on page-locked host x/y, each copying x in, "
                        "running the SpMV and copying y out, consecutive calls overlapping (copies in, compute, "
                        "copies out on three streams); wall clock from first enqueue to SpB_VNEC_host_wait_ext; "
                        f"the plan's device arrays ({info.device_bytes / 1e9:.1f} GB) exceed L2",
                "sync_value": round(e2e_value, 3), "sync_steps": e2e_steps,
                "sync_path": "SpB_mxv_host_ext, one blocking call per step (H2D x, SpMV in row-window parts, "
                             "D2H y per part), L2 flushed before each call"},
        "gpu_launches": args.steps * info.launches_per_call,
        "clocks": clocks,
        "rel_error": {"max_rowwise": float(rel.max()), "median_rowwise": float(np.median(rel)),
                      "criterion": f"|y-yhat| <= {PREC_TOL[args.precision]:g} * sum|a x| (compensated FP64 oracle)"},
    }
    if not args.no_legs:
        legs = {args.workload: form_legs(m, xv, B, flush, stream, args.leg_steps, args.warmup)}
        if args.workload == "rmat24":
            m2, x2, _ = workload("stencil256")
            legs["stencil256"] = form_legs(m2, x2, algorithmic_bytes(m2), flush, stream, args.leg_steps, args.warmup)
            m2.free()
        line["legs"] = legs
        if args.workload == "rmat24":
            line["tuner_live"] = tuner_live_leg()
        if args.workload in ("rmat24", "rmat22"):
            line["gather_ceiling"] = gather_ceiling_leg(m, x, flush, stream, float(np.mean(main_ms)))
        if args.workload == "rmat24" and not args.no_batch_leg:
            from vnec_gb300 import generators as G

            mats = G.batch_lognormal(512, seed=0)
            blegs, _, _ = batch_legs(mats, [1, 32], [api.PREC_FP64, api.PREC_FP32, api.PREC_DF32], 5, args.warmup,
                                     dev, flush, stream, ws)
            line["batch_legs"] = {"workload": BATCH_DESC, "legs": blegs}
            for m3 in mats:
                m3.free()
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        secs, reps, sample, kind = cpu_time_L(m, xv, warm=1, reps=40, budget_s=args.cpu_budget)
        cores, _, _ = reference_cores_and_parts()
        line["cpu_baseline"] = {"value": round(B / secs / 1e9, 3), "unit": "GB/s", "cores": cores, "kind": kind,
                                "sample": f"full workload, 1 warm-up + {reps} calls; {sample}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.free()
    if ws > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# Batched multi-right-hand-side workload.
# ---------------------------------------------------------------------------

BATCH_DESC = ("512 square CSR matrices, rows log-uniform in [1e3, 2e5], row lengths lognormal(ln 8, 1.5) capped "
              "at 4096, uniform distinct columns, values U(-1,1) FP64, seed 0; X row-major FP64 U(-1,1)")
FP64_PEAK_TFLOPS = 1.25  # nominal GB300 FP64 (non-tensor) rate


def batch_bytes(nnz: int, n_rows: int, n_cols: int, n_mats: int, k: int, vb: int = 8) -> int:
    return nnz * (vb + 4) + (n_rows + n_mats) * 4 + (n_rows + n_cols) * k * 8


def batch_legs(mats, ks, precs, steps: int, warmup: int, dev, flush, stream, ws: int = 1, tile=None):
    """Every (precision, k) of the batched form on `mats`: autotuned plan, graph
    replays timed with CUDA events (L2 flushed before each), end-to-end host
    calls and error on every 32nd matrix.  Returns (legs, launches, first leg)."""
    import torch

    from oracle import oracle as O
    from vnec_gb300 import api

    nnz = sum(m.nnz for m in mats)
    n_rows = sum(m.n_rows for m in mats)
    n_cols = sum(m.n_cols for m in mats)
    peak, _ = measured_peaks()
    legs = {}
    gpu_launches = 0
    first = None
    rng = np.random.default_rng(1)
    for prec in precs:
        for k in ks:
            t_plan = time.time()
            if tile:  # fixed layout (lanes, long-row limit, warps per block, unroll), no autotune
                plan = api.BatchPlan(mats, k, precision=prec, lanes=tile[0], long_row_len=tile[1],
                                     warps_per_block=tile[2], unroll=tile[3],
                                     dispatch=tile[4] if len(tile) > 4 else 0, k1_layout=-1)
            else:
                plan = api.BatchPlan(mats, k, precision=prec, autotune=True)
            t_plan = time.time() - t_plan
            info = plan.info()
            ro, co = plan.offsets()
            xv = rng.uniform(-1, 1, n_cols * k)
            x = torch.from_numpy(xv).to(dev)
            y = torch.empty(n_rows * k, dtype=torch.float64, device=dev)
            B = batch_bytes(nnz, n_rows, n_cols, len(mats), k, 4 if prec == api.PREC_FP32 else 8)
            pname = {api.PREC_FP64: "fp64", api.PREC_FP32: "fp32", api.PREC_DF32: "df32"}[prec]
            with torch.cuda.stream(stream):
                for _ in range(warmup):
                    flush.fill_(1)
                    plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
            stream.synchronize()
            starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
            ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
            if ws > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                for i in range(steps):
                    flush.fill_(i)
                    starts[i].record(stream)
                    plan.mxv_device(x.data_ptr(), y.data_ptr(), stream.cuda_stream)
                    ends[i].record(stream)
            torch.cuda.synchronize()
            ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
            total = replica_max(float(np.sum(ms)), dev)
            gpu_launches += steps * info.launches_per_call
            value = replica_throughput(B, steps, ws, total)
            # end to end: pinned host X / Y through SpB_mxv_host_ext
            hx = torch.from_numpy(xv).pin_memory()
            hy = torch.empty(n_rows * k, dtype=torch.float64).pin_memory()
            plan.mxv_host(hx.numpy(), hy.numpy())
            e2e_steps = max(1, steps // 4)
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                plan.mxv_host(hx.numpy(), hy.numpy())
            e2e_s = time.perf_counter() - t0
            # Enough calls that filling and draining the three-stage pipeline
            # (one x copy in, one y copy out) does not dominate the rate.
            pipe_steps = max(16, steps // 4)
            pipe_s, hy_pipe = pipelined_e2e(plan, hx.numpy(), n_rows * k, pipe_steps)
            y_dev = y.cpu().numpy()
            if not np.array_equal(hy.numpy(), y_dev) or not np.array_equal(hy_pipe, y_dev):
                raise RuntimeError("host-path and device-path batch results differ")
            errs = []
            for i in range(0, len(mats), max(1, len(mats) // 16)):
                m = mats[i]
                Yr, cond = O.spmm_neumaier(m, xv[co[i] * k:co[i + 1] * k].reshape(m.n_cols, k))
                Yg = y_dev[ro[i] * k:ro[i + 1] * k].reshape(m.n_rows, k)
                errs.append(O.rowwise_error(Yg, Yr, cond).ravel())
            rel = np.concatenate(errs)
            cand, tms, best = plan.tuning()
            mean_ms = total / steps
            leg = {"k": k, "precision": pname,
                   "gbs": round(value, 2), "ms_per_step": round(mean_ms, 4),
                   "hbm_frac": round(B / (mean_ms / 1e3) / 1e9 / peak, 4),
                   "fp64_tflops": round(2 * nnz * k / (mean_ms / 1e3) / 1e12, 4),
                   "e2e_gbs": round(B * pipe_steps / pipe_s / 1e9, 2),
                   "e2e_sync_gbs": round(B * e2e_steps / e2e_s / 1e9, 2),
                   "h2d_bytes_per_step": n_cols * k * 8, "d2h_bytes_per_step": n_rows * k * 8,
                   "algorithmic_bytes": B,
                   "layout": ("one sliced row-group plan of the block-diagonal concatenation (k = 1), unroll "
                              f"{info.items_per_thread}" if info.lanes == 0 else "batch kernel"),
                   "lanes": info.lanes, "long_row_len": info.long_row_len,
                   "threads_per_block": info.threads_per_block, "tasks": info.num_tiles,
                   "tuner": {"candidates": len(cand), "best_ms_on_sample": round(tms[best], 4) if cand else None,
                             "worst_ms_on_sample": round(max(tms), 4) if cand else None,
                             "chosen": list(cand[best]) if cand else None},
                   "plan_build_s": round(t_plan, 2), "launches_per_call": info.launches_per_call,
                   "rel_error": {"max": float(rel.max()), "median": float(np.median(rel))}}
            legs[f"{pname}_k{k}"] = leg
            if first is None:
                first = (leg, B)
            plan.free()
            del x, y, hx, hy
            torch.cuda.empty_cache()
    for leg in legs.values():
        base = legs.get(f"fp64_k{leg['k']}")
        if base:
            leg["speedup_vs_fp64"] = round(base["ms_per_step"] / leg["ms_per_step"], 3)
    return legs, gpu_launches, first


def run_batch(args) -> None:
    import torch

    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    t_gen = time.time()
    mats = G.batch_lognormal(args.batch_mats, seed=0)
    t_gen = time.time() - t_gen
    nnz = sum(m.nnz for m in mats)
    n_rows = sum(m.n_rows for m in mats)
    n_cols = sum(m.n_cols for m in mats)
    ks = [int(v) for v in args.rhs.split(",")]
    precs = [{"fp64": api.PREC_FP64, "fp32": api.PREC_FP32, "df32": api.PREC_DF32}[p]
             for p in args.batch_precision.split(",")]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    peak, peak_src = measured_peaks()
    sampler = ClockSampler(dev.index)
    w0 = time.time()
    tile = [int(v) for v in args.batch_tile.split(",")] if args.batch_tile else None
    legs, gpu_launches, first = batch_legs(mats, ks, precs, args.batch_steps, args.warmup, dev, flush, stream, ws,
                                           tile=tile)
    w1 = time.time()
    clocks = sampler.stop(w0, w1)
    leg, B = first
    line = {
        "metric": METRIC, "value": leg["gbs"], "unit": "GB/s", "n_gpus": ws, "steps": args.batch_steps,
        "warmup": args.warmup, "ms_per_step": leg["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp32": "f32 (fp64 reductions)", "df32": "f32 hi+lo (double-float)"}[leg["precision"]],
        "data": "synthetic (seeded generator, resident in HBM before timing)",
        "config": {"workload": "batch512_lognormal_" + leg["precision"] + f"_k{leg['k']}", "desc": BATCH_DESC,
                   "n_mats": len(mats), "n_rows": n_rows, "n_cols": n_cols, "nnz": nnz, "k": leg["k"],
                   "l2": "flushed before every timed step (512 MiB device write, outside the events)",
                   "graph": "one CUDA graph replay per step (persistent kernel)", "gen_s": round(t_gen, 2)},
        "roofline": {"bound": "hbm", "kernel": "batch_kernel", "achieved": round(B / (leg["ms_per_step"] / 1e3) / 1e9, 1),
                     "peak": peak, "unit": "GB/s", "frac": leg["hbm_frac"], "peak_source": peak_src,
                     "traffic": None, "fp64_tflops": leg["fp64_tflops"], "fp64_peak_tflops": FP64_PEAK_TFLOPS,
                     "fp64_frac": round(leg["fp64_tflops"] / FP64_PEAK_TFLOPS, 4)},
        "e2e": {"value": leg["e2e_gbs"], "unit": "GB/s", "h2d_bytes_per_step": leg["h2d_bytes_per_step"],
                "d2h_bytes_per_step": leg["d2h_bytes_per_step"],
                "path": "SpB_mxv_host_async_ext on a batch plan: independent calls on page-locked host X/Y, "
                        "consecutive calls overlapping copies in, compute and copies out",
                "sync_value": leg["e2e_sync_gbs"],
                "sync_path": "SpB_mxv_host_ext on a batch plan, one blocking call per step"},
        "gpu_launches": gpu_launches, "clocks": clocks, "legs": legs,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = batch_cpu_baseline(mats, leg["k"], args.cpu_budget)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def batch_cpu_baseline(mats, k: int, budget_s: float) -> dict:
    """The reference's way to run a batch: SpMV_VNEC_L_FP64 per matrix and per
    right-hand side (oracle port), timed on a sample of the matrices."""
    from oracle import oracle as O

    cores, nparts, arch = reference_cores_and_parts()
    rng = np.random.default_rng(3)
    order = np.argsort([m.nnz for m in mats])
    pick = [mats[i] for i in order[::max(1, len(mats) // 32)]]
    t_total, B_total, calls = 0.0, 0, 0
    t_start = time.time()
    own = O.ref_available()
    for m in pick:
        x = rng.uniform(-1, 1, m.n_cols)
        t = O.ref_time_f64(m, x, 3, warm=1, reps=3)[0] if own else O.time_L_f64(m, x, nparts, warm=1, reps=3)
        t_total += t * k
        B_total += batch_bytes(m.nnz, m.n_rows, m.n_cols, 1, k)
        calls += 4
        if time.time() - t_start > budget_s:
            break
    what = "the reference's own SpMV_VNEC_L_FP64 (its build for this host)" if own else \
        "SpMV_VNEC_L_FP64 restated (oracle port)"
    return {"value": round(B_total / t_total / 1e9, 3), "unit": "GB/s", "cores": cores,
            "kind": "reference" if own else "port",
            "sample": f"{len(pick)} of {len(mats)} matrices (evenly spaced in nnz order), {what} per matrix, "
                      f"1 warm-up + 3 timed calls, x {k} right-hand sides; {nparts} OpenMP threads on {cores} "
                      f"{arch} cores"}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="rmat24",
                    choices=["rmat24", "rmat22", "uniform64k", "stencil256", "stencil128", "batch512"])
    ap.add_argument("--rhs", default="1,4,8,16,32", help="batch512: right-hand-side counts")
    ap.add_argument("--batch-precision", default="fp64", help="batch512: fp64,fp32")
    ap.add_argument("--batch-mats", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--batch-tile", default="", help="batch512: fixed lanes,long_row_len,warps_per_block,unroll"
                                                     "[,dispatch: 1 persistent warps, 2 one warp per task] "
                                                     "instead of the autotuner")
    ap.add_argument("--kernel", default="S", choices=["L", "S", "D"])
    ap.add_argument("--l2", default="flushed", choices=["flushed", "warm"],
                    help="flush L2 before each timed step (default) or keep it warm (small workloads' warm figure)")
    ap.add_argument("--precision", default="fp64", choices=list(PRECISIONS),
                    help="sliced-kernel form of the main plan (the headline is fp64)")
    ap.add_argument("--shared-patterns", default="on", choices=["on", "off"],
                    help="precision forms: one copy of the column gaps for row groups that share them (default on)")
    ap.add_argument("--unroll", type=int, default=-1, choices=[-1, 4, 8, 12, 16],
                    help="sliced plans: loads in flight per lane (-1: timed on the matrix at plan build)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-legs", action="store_true", help="skip the precision-form / tuner / batch legs")
    ap.add_argument("--no-batch-leg", action="store_true", help="skip the batched-form legs of the default run")
    ap.add_argument("--leg-steps", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU-baseline timing")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    # Thread placement of the reference's own run script (run_vnec.sh:8-9),
    # for the CPU legs of both arms (set before any OpenMP runtime starts).
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch512":
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
