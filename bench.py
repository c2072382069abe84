#!/usr/bin/env python
"""bench.py — HS-field updates/s of the DQMC sweep on GB300.

Metric (the reference's sweep counting, src/dqmc.cpp:88-92): HS-field update
attempts per second = walkers * N * Lt / half-sweep time, of the batched
mixed-precision sweep against the FP64 path, with the mixed path's max |dG|
against FP64 on the same fields.  One step = one half-sweep (alternating
0->beta and beta->0) of every walker, equal-time measurement fused.  Default
workload: 128 walkers, attractive Hubbard 16x16 (N=256), t=1, |U|=4,
mu=-0.5, beta=10, dtau=0.1 (Lt=100), dense exp(-dtau K), stabilization every
8 slices, seeded +/-1 fields; wraps, B-chain and stabilization products on the
tensor cores (exact-slice BF16, tcgen05), FP64 elsewhere.  For this workload
the line also carries the FP64 batch on the same configuration, the plain
single-walker FP64 path, and max |dG| at every stabilization of a half-sweep
(mixed against FP64 on the same fields and uniforms, a sample of walkers).

Legs printed on one JSON line:
  value        device-timed throughput (CUDA events on the library's stream,
               inputs resident in HBM, Philox uniforms on the device)
  e2e          the same metric through the C-ABI in reference-RNG mode: the
               host draws each walker's minstd_rand0 uniforms, copies them in
               (pinned -> HBM), runs the half-sweep and reads every walker's
               observable accumulators back, all inside the timed region
  roofline     the dominant kernel class: its algorithmic flops over its CUDA-event
               time in profiled replays of the same half-sweeps, against the FP64
               FMA rate measured on this device (FP64 classes) or the measured bf16
               rate (tensor-core classes); DRAM traffic per launch from ncu
  cpu_baseline the CPU oracle (reference algorithm restated, scipy LAPACK),
               one walker per host core, on a bounded sample

--impl reference times only the CPU restatement of the reference (all host
cores), with the same metric and workload.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))

WORKLOADS = {
    # batch of 256 FP64 walkers, checkerboard (the batched FP64 configuration)
    "fp64_batch_8x8_checkerboard": dict(walkers=256, model=0, L=8, U=4.0, mu=0.0, beta=8.0, Lt=160, pace=10,
                                         checkerboard=True),
    # 128 FP64 walkers, attractive 16x16 dense, beta=10 (the plain-FP64 run of the
    # mixed-precision configuration: same model, lattice, beta and pace)
    "fp64_batch_16x16_attractive": dict(walkers=128, model=1, L=16, U=4.0, mu=-0.5, beta=10.0, Lt=100, pace=8,
                                        checkerboard=False),
    # the mixed-precision configuration: 128 walkers, attractive 16x16 (U=-4 as |U|=4
    # on the attractive model), mu=-0.5, beta=10, dtau=0.1, wraps and B-chain on the
    # tensor cores, FP64 stabilization every 8 slices
    "mixed_batch_16x16_attractive": dict(walkers=128, model=1, L=16, U=4.0, mu=-0.5, beta=10.0, Lt=100, pace=8,
                                         checkerboard=False, precision="mixed"),
    # one FP64 walker, 4x4 dense (the reference's single-chain case)
    "fp64_single_4x4_dense": dict(walkers=1, model=0, L=4, U=4.0, mu=0.0, beta=4.0, Lt=80, pace=10,
                                  checkerboard=False),
}
DEFAULT_WORKLOAD = "mixed_batch_16x16_attractive"
METRIC = "HS-field updates/s (walkers*N*Lt / half-sweep time)"


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant
# kernel of a class on the tensor-core path, from one ncu --set full capture each of an
# 8-walker launch of the 16x16, beta = 10 configuration.  ncu replays a kernel with L2
# flushed, and each walker's G, chain and slices are its own, so this cold-cache traffic
# grows in proportion to the walkers a launch covers.
NCU_TRAFFIC_8_WALKERS = {
    "metropolis": ("metropolis_sub_kernel", 4436480 + 256),
    "product": ("oz_prod_tc_kernel<3,7>", 8307200 + 0),
}


def ncu_traffic(workload: dict, cls: str, walkers_per_launch: int):
    """(bytes per launch, kernel, how it was obtained) of a class's dominant kernel, scaled
    from the 8-walker capture, or (None, None, reason) where no capture covers the class."""
    if workload.get("precision") != "mixed" or workload["L"] != 16 or cls not in NCU_TRAFFIC_8_WALKERS:
        return None, None, "no ncu capture of this class for this workload"
    kern, b8 = NCU_TRAFFIC_8_WALKERS[cls]
    return b8 * walkers_per_launch / 8, kern, (
        f"ncu --set full capture of {kern} on an 8-walker launch (L2 flushed), scaled to the "
        f"{walkers_per_launch} walkers of one profiled launch")


L2_BYTES = 129 * 2 ** 20


def working_set_bytes(wl: dict) -> int:
    """Device bytes one timed step touches per GPU, a lower bound: each walker's G (both
    spins), B-chain and the two UDT stacks (U, F and D per level and spin)."""
    N, S = wl["L"] ** 2, (1 if wl["model"] == 1 else 2)
    ns = -(-wl["Lt"] // wl["pace"])
    per = 8 * (2 * N * N + S * N * N + 2 * S * ns * (2 * N * N + N))
    return wl["walkers"] * per


def l2_note(wl: dict) -> str:
    ws = working_set_bytes(wl)
    if ws > L2_BYTES:
        return (f"no flush: the per-GPU working set (G, chains, UDT stacks, >= {ws / 2 ** 30:.2f} GiB) "
                f"is larger than the 129 MB L2")
    return (f"no flush, working set {ws / 2 ** 20:.1f} MiB fits in L2: a latency case, "
            f"not a bandwidth measurement")


def _descs(dq, wl, seed0=1000):
    return [dq.WalkerDesc(model=wl["model"], L=wl["L"], U=wl["U"], mu=wl["mu"], beta=wl["beta"], Lt=wl["Lt"],
                          pace=wl["pace"], checkerboard=wl["checkerboard"], seed=seed0 + w)
            for w in range(wl["walkers"])]


# ----------------------------------------------------------------------------
# CPU leg (oracle).  Run in spawned processes: one walker per core.
# ----------------------------------------------------------------------------
def _cpu_walker(args):
    wl, seed, budget_s = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.use_scipy_lapack(True)
    w = O.Walker(model=wl["model"], L=wl["L"], U=wl["U"], mu=wl["mu"], beta=wl["beta"], Lt=wl["Lt"],
                 pace=wl["pace"], checkerboard=wl["checkerboard"], stack=O.STACK_SVD, record=True)
    w.seed(seed)
    w.fields_random()
    w.init()
    w.sweep_0_to_beta()  # warm-up half-sweep
    n, t0 = 0, time.perf_counter()
    while True:
        if n % 2 == 0:
            w.sweep_beta_to_0()
        else:
            w.sweep_0_to_beta()
        w.measure()
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 200:
            break
    return n, el


def cpu_baseline(wl, budget_s=12.0):
    cores = os.cpu_count() or 1
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_walker, [(wl, 5000 + c, budget_s) for c in range(cores)])
    wall = time.perf_counter() - t0
    upd = wl["L"] ** 2 * wl["Lt"]
    per_core = [n * upd / el for n, el in res]
    agg = sum(per_core)
    sample = (f"{cores} independent oracle walkers (reference SVD-stack algorithm, scipy LAPACK, "
              f"1 thread each), {min(n for n, _ in res)}-{max(n for n, _ in res)} measured half-sweeps "
              f"each of {wl['L']}x{wl['L']}, Lt={wl['Lt']}, {budget_s:.0f} s budget; wall {wall:.1f} s")
    return {"value": agg, "unit": "updates/s", "cores": cores, "kind": "port", "sample": sample,
            "per_core": statistics.mean(per_core)}


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None
        self.path = None

    def start(self):
        try:
            # samples go to DQMC_BENCH_CLOCKS_DIR when set (to keep them), else a temporary file
            d = os.environ.get("DQMC_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
            os.makedirs(d, exist_ok=True)
            self.path = os.path.join(d, f"dqmc_bench_clocks_{os.getpid()}.csv")
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------
# algorithmic work per walker per half-sweep: the reference's sweep, counted as it executes
# ----------------------------------------------------------------------------
def flops_model(wl, accepts_per_walker_per_half):
    N, Lt, p = wl["L"] ** 2, wl["Lt"], wl["pace"]
    S = 1 if wl["model"] == 1 else 2
    ns = -(-Lt // p)
    if wl["checkerboard"]:
        W, C = 34 * N * N, 17 * N * N
    else:
        W, C = 4 * N ** 3 + 2 * N * N, 2 * N ** 3 + N * N
    seg = S * Lt * (W + C) + S * accepts_per_walker_per_half * 2 * N * N
    # stabilization counted as executed by this path (column-pivoted QR):
    # push = QR 4/3 N^3 + forming Q 4/3 N^3 + triangular T F_prev N^3;
    # greens = U_L^T U_R, F_L F_R^T (4 N^3) + LU 2/3 N^3 + solve 2 N^3 + final GEMM 2 N^3
    push = S * ns * (8.0 / 3.0 + 1.0) * N ** 3
    greens = S * ns * (4.0 + 2.0 / 3.0 + 2.0 + 2.0) * N ** 3
    nominal = S * Lt * (W + C) + S * accepts_per_walker_per_half * 2 * N * N + S * ns * 33 * N ** 3
    return {"segment": seg, "push": push, "greens": greens, "nominal_F": nominal}


def stab_tensor_flops(N, TB=32):
    """FP64-equivalent flops of the tensor-core products of one push and one
    Green's assembly (blocked Householder, panel TB), per walker and spin."""
    push = 2 * N ** 3  # F = D^-1 R P^T F_prev
    greens = 3 * 2 * N ** 3  # M = ... U_L^T U_R ..., += F_L F_R^T, G = U_R X
    for p in range(-(-N // TB)):
        j0 = p * TB
        m = N - j0
        pb = min(TB, m)
        nt = m - pb
        qr = (2 * pb * nt * m + 2 * pb * nt * pb + 2 * m * nt * pb) if nt > 0 else 0
        push += qr + 2 * pb * m * m + 2 * pb * m * pb + 2 * m * m * pb  # trailing update, forming Q
        greens += qr + 2 * pb * N * m + 2 * pb * N * pb + 2 * m * N * pb  # trailing update, Q^T Y
        if j0 + pb < N:
            greens += 2 * pb * N * (N - j0 - pb)  # block back substitution
    return push, greens


def observable_deviation(mixed, fp64, names, write_bin):
    """Each equal-time observable of the mixed path against the FP64 path run on the same
    fields and uniforms: |mean over walkers (mixed) - mean (FP64)| in units of the standard
    error of the FP64 walkers' mean.  mixed, fp64: (sums, counts) per walker as
    observables_all returns them; write_bin normalises one walker's bin."""
    import numpy as np

    vm = np.array([write_bin(s, c) for s, c in zip(*mixed)])
    vf = np.array([write_bin(s, c) for s, c in zip(*fp64)])
    n = len(vf)
    out = {}
    for k, name in enumerate(names):
        d = float(abs(vm[:, k].mean() - vf[:, k].mean()))
        se = float(vf[:, k].std(ddof=1) / np.sqrt(n)) if n > 1 else 0.0
        out[name] = {"abs_diff": d, "fp64_stderr": se, "in_stderr": d / se if se > 0 else None}
    return out


def fp64_comparison(args, dq, wl, stream, sample=8):
    """The FP64 path on the same configuration (throughput), the plain
    single-walker FP64 path, and max |dG| of the mixed path against FP64 at
    every stabilization of one half-sweep on the same fields and uniforms."""
    import torch

    def timed_rate(descs, steps):
        b = dq.Batch(descs, rng=dq.RNG_PHILOX, precision=dq.FP64)
        b.set_stream(stream.cuda_stream)
        for w in range(len(descs)):
            b.fields_random(w)
        b.init_greens()
        b.sweep_0_to_beta(measure=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(steps):
            (b.sweep_beta_to_0 if k % 2 == 0 else b.sweep_0_to_beta)(measure=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        upd = b.updates_per_half_sweep()
        b.close()
        return upd * steps / (ms * 1e-3), ms / steps

    descs = _descs(dq, wl)
    fp64_value, fp64_ms = timed_rate(descs, 2)
    single_value, single_ms = timed_rate(descs[:1], 1)
    # accuracy gate on a sample of walkers: identical decisions, |dG| at every stabilization
    sub = descs[:sample]
    traces, fields, obs = [], [], []
    for prec in (dq.MIXED, dq.FP64):
        b = dq.Batch(sub, rng=dq.RNG_PHILOX, precision=prec, trace=True)
        for w in range(len(sub)):
            b.fields_random(w)
        b.init_greens()
        b.sweep_0_to_beta(measure=True)
        traces.append([b.trace(w) for w in range(len(sub))])
        fields.append([b.fields(w) for w in range(len(sub))])
        obs.append(b.observables_all())
        b.close()
    same = [bool((fields[0][w] == fields[1][w]).all()) for w in range(len(sub))]
    dg = max(float(abs(traces[0][w] - traces[1][w]).max()) for w in range(len(sub)) if same[w]) if any(same) else None
    try:
        dev = observable_deviation(obs[0], obs[1], dq.OBS_NAMES, dq.write_bin)
        worst = max((v["in_stderr"] for v in dev.values() if v["in_stderr"] is not None), default=None)
    except Exception as e:  # the throughput line must not depend on this report
        dev, worst = {"unavailable": f"{type(e).__name__}: {e}"}, None
    return {"fp64_batch_value": fp64_value, "fp64_batch_ms_per_step": fp64_ms,
            "fp64_single_walker_value": single_value, "fp64_single_walker_ms_per_step": single_ms,
            "max_abs_dG": dg, "dG_sample": f"{len(sub)} walkers, every stabilization of one 0->beta half-sweep, "
                                            f"same fields and Philox uniforms",
            "walkers_with_identical_decisions": int(sum(same)),
            "observables_vs_fp64": dev, "max_observable_dev_in_stderr": worst}


def run_gpu(args, wl, rank, world):
    import torch

    import dqmc_gb300 as dq

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    fp64_peak = dq.microbench_fp64()

    descs = _descs(dq, wl, seed0=1000 + 100000 * rank)
    prec = dq.MIXED if wl.get("precision") == "mixed" else dq.FP64
    batch = dq.Batch(descs, rng=dq.RNG_PHILOX, precision=prec)
    # a dedicated stream: the library launches on it and the CUDA events below
    # are recorded on it (torch's default stream would be handle 0)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    batch.set_stream(stream.cuda_stream)
    for w in range(len(descs)):
        batch.fields_random(w)
    batch.init_greens()
    upd = batch.updates_per_half_sweep()
    tuning = batch.tuning()

    def step(k, b=batch):
        if k % 2 == 0:
            b.sweep_0_to_beta(measure=True)
        else:
            b.sweep_beta_to_0(measure=True)

    for k in range(args.warmup):
        step(k)
    acc0 = sum(batch.accept_count(w) for w in range(len(descs)))
    launches0 = batch.launch_count()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")  # lets a profiler select exactly the timed steps
    e0.record(stream)
    for k in range(args.steps):
        step(args.warmup + k)
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    acc1 = sum(batch.accept_count(w) for w in range(len(descs)))
    launches = batch.launch_count() - launches0
    # per-kernel-class CUDA-event times: the same number of half-sweeps replayed again
    # as profiled graphs (event nodes around each class, one branch), after the timed region
    batch.profile_enable(True)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for k in range(args.steps):
        step(args.warmup + args.steps + k)
    p1.record(stream)
    torch.cuda.synchronize()
    prof_total = p0.elapsed_time(p1)
    prof = batch.profile_read()
    batch.profile_enable(False)
    status = [batch.status(w) for w in range(len(descs))]
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * upd * args.steps / (ms * 1e-3)

    # ---- roofline of the dominant kernel class (algorithmic work of the class / its CUDA-event time)
    acc_per_walker_half = (acc1 - acc0) / len(descs) / args.steps
    fm = flops_model(wl, acc_per_walker_half)
    N, S, Lt = wl["L"] ** 2, (1 if wl["model"] == 1 else 2), wl["Lt"]
    ns = -(-Lt // wl["pace"])
    units = len(descs) * args.steps  # walker half-sweeps in the timed region
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    bf16_peak = peaks.get("bf16_tflops_sustained") or 1700.0
    bf16_src = ("MEASURED_PEAKS.json bf16_tflops_sustained (the class runs inside a long step)"
                if "bf16_tflops_sustained" in peaks else "fallback 1.7 PFLOP/s sustained bf16")
    fp64_src = "FP64 FMA probe measured in this run (dqmc_microbench_fp64); MEASURED_PEAKS.json holds no FP64 figure"
    model = {}  # class -> (bound, algorithmic flops in the timed region, peak TFLOP/s, what is counted)
    if wl.get("precision") == "mixed":
        sl = 6 * 7 // 2 if N <= 256 else 7 * 8 // 2  # slice products of one wrap or chain product
        model["product"] = ("tensor", units * S * Lt * 3 * sl * 2 * N ** 3, bf16_peak,
                            f"BF16 flops of the exact-slice products: 3 per slice x {sl} slice pairs x 2N^3")
        if N >= 128:
            pf, gf = stab_tensor_flops(N)
            pairs = 36 if N <= 256 else 45
            model["push"] = ("tensor", units * S * ns * pf * pairs, bf16_peak,
                             f"BF16 flops of the blocked-QR products ({pairs} slice pairs per FP64-class product)")
            model["greens"] = ("tensor", units * S * ns * gf * pairs, bf16_peak,
                               f"BF16 flops of the Green's-assembly products ({pairs} slice pairs)")
        model["metropolis"] = ("fp64", units * S * acc_per_walker_half * 2 * N * N, fp64_peak / 1e3,
                               "the reference's rank-1 update flops, 2 N^2 per accepted flip and spin")
    else:
        for k in ("segment", "push", "greens"):
            model[k] = ("fp64", fm[k] * units, fp64_peak / 1e3, "FP64 flops of the class (flops_model: wraps, chain products, Green's assembly)")
    dom = max((k for k in model if prof.get(k, (0, 0))[1] > 0), key=lambda k: prof[k][0])
    bound, flops, peak, what = model[dom]
    dom_ms, dom_n = prof[dom]
    achieved = flops / (dom_ms * 1e-3) / 1e12
    # the profiled replay runs one branch, so each of its launches covers every walker
    traffic, traffic_kernel, traffic_src = ncu_traffic(wl, dom, len(descs))
    roofline = {"bound": bound, "kernel": f"{dom} kernel class", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                "traffic_kernel": traffic_kernel, "traffic_source": traffic_src,
                "peak_source": bf16_src if bound == "tensor" else fp64_src, "counted": what,
                "avg_launch_ms": dom_ms / max(dom_n, 1),
                "kernel_share": {k: prof[k][0] / prof_total for k in prof if prof[k][1] > 0},
                "profiled_ms_per_step": prof_total / args.steps,
                "classes": {k: {"bound": v[0], "achieved_tflops": v[1] / (prof[k][0] * 1e-3) / 1e12,
                                "frac": v[1] / (prof[k][0] * 1e-3) / 1e12 / v[2]}
                            for k, v in model.items() if prof.get(k, (0, 0))[0] > 0},
                "sweep_nominal_F_tflops": fm["nominal_F"] * units / (ms * 1e-3) / 1e12}

    # ---- e2e: reference RNG on the host, copies in and out every step
    e2e = None
    if rank == 0 or world > 1:
        eb = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec)
        eb.set_stream(stream.cuda_stream)
        for w in range(len(descs)):
            eb.fields_random(w)
        eb.init_greens()
        for k in range(max(1, min(args.warmup, 3))):
            step(k, eb)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        ek = max(2, min(args.steps, 10))
        for k in range(ek):
            step(k, eb)
            sums, counts = eb.observables_all()
        el = time.perf_counter() - t0
        barrier()
        e2e = {"value": world * upd * ek / el, "unit": "updates/s",
               "h2d_bytes_per_step": 8 * upd, "d2h_bytes_per_step": int(sums.nbytes + counts.nbytes),
               "steps": ek, "rng": "host minstd_rand0 (reference stream)"}
        eb.close()
    cmp = None
    if wl.get("precision") == "mixed" and rank == 0 and world == 1 and not args.no_compare:
        cmp = fp64_comparison(args, dq, wl, stream)
    return dict(value=value, ms=ms, roofline=roofline, e2e=e2e, clocks=clk, launches=launches, status=status,
                tuning=tuning, fp64=cmp,
                accept_rate=acc_per_walker_half / (wl["L"] ** 2 * wl["Lt"]), fp64_peak=fp64_peak)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the FP64 comparison legs (profiling runs)")
    ap.add_argument("--walkers", type=int, default=0, help="override the walker count (profiling runs)")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload])
    if args.walkers > 0:
        wl["walkers"] = args.walkers
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    config = {"workload": args.workload, "walkers_per_gpu": wl["walkers"], "model": "repulsive" if wl["model"] == 0 else "attractive",
              "L": wl["L"], "N": wl["L"] ** 2, "U": wl["U"], "mu": wl["mu"], "beta": wl["beta"], "Lt": wl["Lt"],
              "pace": wl["pace"], "expK": "checkerboard" if wl["checkerboard"] else "dense",
              "precision": wl.get("precision", "fp64"),
              "measure": "equal-time, fused", "parallelism": f"replicas x{args.gpus}",
              "l2": l2_note(wl)}

    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_baseline(wl, budget_s=max(4.0, args.cpu_budget))
        steps = args.steps
        line = {"metric": METRIC, "value": cb["value"], "unit": "updates/s", "n_gpus": args.gpus, "steps": steps,
                "warmup": args.warmup, "ms_per_step": wl["walkers"] * wl["L"] ** 2 * wl["Lt"] / cb["value"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded +/-1 fields)", "config": config, "impl": "reference",
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cb["value"], "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        line["cpu_baseline"]["kind"] = "port"
        print(json.dumps(line))
        return

    r = run_gpu(args, wl, rank, world)
    if rank != 0:
        return
    cb = None
    if world == 1 and not args.no_cpu:
        cb = cpu_baseline(wl, budget_s=args.cpu_budget)
        cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    line = {"metric": METRIC, "value": r["value"], "unit": "updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64; products as exact bf16 slices" if wl.get("precision") == "mixed" else "f64",
            "data": "synthetic (seeded +/-1 fields)",
            "config": config, "roofline": r["roofline"], "cpu_baseline": cb, "e2e": r["e2e"],
            "gpu_launches": r["launches"], "clocks": r["clocks"], "accept_rate": r["accept_rate"],
            "walker_status_nonzero": sum(1 for s in r["status"] if s)}
    if r["tuning"]["candidates"]:
        line["autotune"] = r["tuning"]
    if r["fp64"]:
        c = r["fp64"]
        line["vs_fp64"] = dict(c, ratio_vs_fp64_batch=r["value"] / c["fp64_batch_value"],
                               ratio_vs_fp64_single_walker=r["value"] / c["fp64_single_walker_value"])
    print(json.dumps(line))


if __name__ == "__main__":
    main()
