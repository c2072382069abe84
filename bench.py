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
tensor cores (exact-slice BF16, tcgen05), FP64 elsewhere.  For the tensor-core
workloads the line also carries the FP64 batch on the same configuration, the
plain single-walker FP64 path, and |dG| at every stabilization of a half-sweep
(mixed against FP64 on the same fields and uniforms, a sample of walkers).
Other workloads (--workload): the FP64 batches, the single 4x4 walker, the large
24x24 batch with the time-displaced half-sweep (one step = one measured
forth-and-back pair), and the uneven batch of sides 6-12 with |U| and beta drawn
per walker (walker-weighted throughput of the whole batch, and each side's
batch alone in `per_side`).

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
cores, one walker each), with the same metric and workload: --steps steps per
core, fewer if its time budget runs out first; the line's steps and ms_per_step
are what one core timed.
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
    # the large batch: 32 walkers, repulsive 24x24 (N=576), U=4, mu=0, beta=12, dtau=0.1 (Lt=120),
    # stabilization every 6 slices, tensor-core path (rank-32 submatrix updates); one step is one
    # measured forth-and-back pair of Dqmc::sweep_forth_and_back with dynamic measurement
    # (src/dqmc.cpp:48-70): the time-displaced 0->beta half-sweep with G(k,tau) and the dynamic
    # observables at tau = 0, 10, ..., 110, then the updating beta->0 half-sweep with equal-time
    # measurement.  Only the updating half-sweep attempts flips, so a step counts N * Lt per walker.
    "mixed_batch_24x24_dynamic": dict(walkers=32, model=0, L=24, U=4.0, mu=0.0, beta=12.0, Lt=120, pace=6,
                                      checkerboard=False, precision="mixed", taus=tuple(range(0, 120, 10))),
    # the uneven batch in one launch sequence: 64 repulsive walkers for each side 6, 8, 10, 12
    # (N = 36 ... 144), mu=0, dtau=0.05, pace 10, |U| and beta per walker from std::mt19937_64(7)
    # (dqmc_gb300.workloads.uneven_batch: |U| in [2, 6), beta in {4, 6, 8}, Lt = 80, 120, 160)
    "mixed_uneven_6_to_12": dict(walkers=256, uneven=True, model=0, L=12, U=None, mu=0.0, beta=None, Lt=None,
                                 pace=10, checkerboard=False, precision="mixed"),
}
DEFAULT_WORKLOAD = "mixed_batch_16x16_attractive"
METRIC = "HS-field updates/s (walkers*N*Lt / half-sweep time)"


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant
# kernel of a class on the tensor-core path, from one ncu --set full capture each of an
# 8-walker launch of the 16x16, beta = 10 configuration.  ncu replays a kernel with L2
# flushed, and each walker's G, chain and slices are its own, so this cold-cache traffic
# grows in proportion to the walkers a launch covers.
NCU_TRAFFIC_8_WALKERS = {
    "metropolis": ("metropolis_sub_kernel", 4379392 + 0),
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


def _descs(dq, wl, seed0=1000):
    """The workload's walkers (seeds seed0, seed0 + 1, ...)."""
    if wl.get("uneven"):
        from dqmc_gb300.workloads import uneven_batch

        return uneven_batch(dq, per_size=wl["walkers"] // 4, seed0=seed0)
    return [dq.WalkerDesc(model=wl["model"], L=wl["L"], U=wl["U"], mu=wl["mu"], beta=wl["beta"], Lt=wl["Lt"],
                          pace=wl["pace"], checkerboard=wl["checkerboard"], seed=seed0 + w)
            for w in range(wl["walkers"])]


def _shape(x) -> dict:
    """L, Lt, pace, model, checkerboard of a workload dict or a walker descriptor."""
    if isinstance(x, dict):
        return x
    return dict(L=x.L, Lt=x.Lt, pace=x.pace, model=x.model, checkerboard=x.checkerboard)


def _host_dq():
    import dqmc_gb300 as dq  # descriptors only: no device, no library call

    return dq


def working_set_bytes(wl: dict) -> int:
    """Device bytes one timed step touches per GPU, a lower bound: each walker's G (both
    spins), B-chain and the two UDT stacks (U, F and D per level and spin)."""
    total = 0
    for d in _descs(_host_dq(), wl):
        N, S = d.L ** 2, (1 if d.model == 1 else 2)
        ns = -(-d.Lt // d.pace)
        total += 8 * (2 * N * N + S * N * N + 2 * S * ns * (2 * N * N + N))
    return total


def l2_note(wl: dict) -> str:
    ws = working_set_bytes(wl)
    if ws > L2_BYTES:
        return (f"no flush: the per-GPU working set (G, chains, UDT stacks, >= {ws / 2 ** 30:.2f} GiB) "
                f"is larger than the 129 MB L2")
    return (f"no flush, working set {ws / 2 ** 20:.1f} MiB fits in L2: a latency case, "
            f"not a bandwidth measurement")


# ----------------------------------------------------------------------------
# CPU leg (oracle).  Run in spawned processes: one walker per core.
# ----------------------------------------------------------------------------
def _cpu_walker(args):
    """One oracle walker (the reference's SVD-stack algorithm, scipy LAPACK, one thread):
    one untimed warm-up half-sweep, then timed steps until `steps` are done or the budget
    is spent (at least one).  A step is one measured half-sweep, or with taus one measured
    forth-and-back pair with the dynamic half-sweep.  Returns (steps, seconds, N * Lt)."""
    p, seed, budget_s, steps, taus = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.use_scipy_lapack(True)
    w = O.Walker(model=p["model"], L=p["L"], U=p["U"], mu=p["mu"], beta=p["beta"], Lt=p["Lt"],
                 pace=p["pace"], checkerboard=p["checkerboard"], stack=O.STACK_SVD, record=True)
    w.seed(seed)
    w.fields_random()
    w.init()
    if not taus:
        w.sweep_0_to_beta()  # warm-up half-sweep
    n, t0 = 0, time.perf_counter()
    while True:
        if taus:
            w.sweep_dynamic(list(taus))
            w.sweep_beta_to_0()
            w.measure()
        else:
            if n % 2 == 0:
                w.sweep_beta_to_0()
            else:
                w.sweep_0_to_beta()
            w.measure()
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= steps:
            break
    return n, el, p["L"] ** 2 * p["Lt"]


def _cpu_samples(wl, cores):
    """(walker parameters, taus) per core, and a description of the sample.  The large
    batch's walkers are sampled at beta = 1.2 (Lt = 12, the same N, dtau and pace, tau =
    0 ... 11): the work per slice does not depend on Lt, and a full Lt = 120 pair takes
    minutes on one core.  The uneven batch puts cores / 4 cores on each side, each a walker
    of that side from the same std::mt19937_64 draw."""
    if wl.get("uneven"):
        descs = _descs(_host_dq(), wl)
        per = len(descs) // 4
        out = [(_shape_full(descs[(c % 4) * per + c // 4]), None) for c in range(cores)]
        return out, "walkers of the uneven batch, cores spread evenly over the four sides"
    p = dict(model=wl["model"], L=wl["L"], U=wl["U"], mu=wl["mu"], beta=wl["beta"], Lt=wl["Lt"], pace=wl["pace"],
             checkerboard=wl["checkerboard"])
    if wl.get("taus"):
        dtau = wl["beta"] / wl["Lt"]
        p.update(Lt=12, beta=12 * dtau)
        return [(p, tuple(range(12)))] * cores, (
            f"{wl['L']}x{wl['L']} walkers at beta={12 * dtau:g}, Lt=12 (the workload's N, dtau and pace), "
            f"dynamic half-sweep at tau=0..11 then updating backward half-sweep per step")
    return [(p, None)] * cores, f"{wl['L']}x{wl['L']}, Lt={wl['Lt']} walkers"


def _shape_full(d) -> dict:
    return dict(model=d.model, L=d.L, U=d.U, mu=d.mu, beta=d.beta, Lt=d.Lt, pace=d.pace,
                checkerboard=d.checkerboard)


def cpu_baseline(wl, budget_s=12.0, steps=200):
    """The oracle on every host core, one single-threaded walker per core (the reference runs
    one chain per MPI rank).  Throughput: for a uniform batch the sum of the cores' rates; for
    the uneven batch the rate at which the cores, load-balanced, would finish one step of the
    whole batch, from each side's per-core rate."""
    cores = os.cpu_count() or 1
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    samples, what = _cpu_samples(wl, cores)
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_walker, [(p, 5000 + c, budget_s, steps, taus) for c, (p, taus) in enumerate(samples)])
    wall = time.perf_counter() - t0
    rates = [n * upd / el for n, el, upd in res]
    if wl.get("uneven"):
        by_side = {}
        for (p, _), r in zip(samples, rates):
            by_side.setdefault(p["L"], []).append(r)
        side_rate = {L: statistics.mean(v) for L, v in by_side.items()}
        descs = _descs(_host_dq(), wl)
        work = sum(d.L ** 2 * d.Lt for d in descs)
        secs = sum(d.L ** 2 * d.Lt / side_rate[d.L] for d in descs)  # one core, whole batch
        agg = cores * work / secs
    else:
        agg = sum(rates)
    n_lo, n_hi = min(n for n, _, _ in res), max(n for n, _, _ in res)
    ms = statistics.mean(el / n for n, el, _ in res) * 1e3
    sample = (f"{cores} independent oracle walkers (reference SVD-stack algorithm, scipy LAPACK, "
              f"1 thread each) of {what}; {n_lo}-{n_hi} timed steps each in a {budget_s:.0f} s budget; "
              f"wall {wall:.1f} s")
    return {"value": agg, "unit": "updates/s", "cores": cores, "kind": "port", "sample": sample,
            "per_core": statistics.mean(rates), "steps": n_lo, "ms_per_step": ms}


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
    """FP64 work of one walker's half-sweep (a workload dict or a walker descriptor), counted
    as the reference's sweep executes it (dqmc_walker.cpp:246-412)."""
    wl = _shape(wl)
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


def stab_rhs_flops(N, TB=32):
    """FP64-equivalent flops of the products that carry one more right-hand side through the
    Green's assembly's factorization (Q^T applied panel by panel, blocked back substitution),
    per walker and spin: the second right-hand side of the dynamic half-sweep."""
    f = 0
    for p in range(-(-N // TB)):
        j0 = p * TB
        m = N - j0
        pb = min(TB, m)
        f += 2 * pb * N * m + 2 * pb * N * pb + 2 * m * N * pb
        if j0 + pb < N:
            f += 2 * pb * N * (N - j0 - pb)
    return f


def slice_pairs(n_slices: int) -> int:
    """Slice products of one exact-slice product: pairs (i, j) with i + j < S."""
    return n_slices * (n_slices + 1) // 2


def wrap_slices(N: int) -> int:
    """Slices of the wraps and B-chain products (ozaki::cfg_for_k): 7 of 7 bits for N <= 256,
    8 of 6 bits above."""
    return 7 if N <= 256 else 8


def block_accepts_sq(p_acc: float, kb: int = 32) -> float:
    """E[m^2] of the accepts m of one 32-site block, m ~ Binomial(32, p)."""
    return kb * p_acc * (1 - p_acc) + (kb * p_acc) ** 2


def metropolis_work(d, accepts: float, tc_flush: int, kd: int):
    """Work one walker's Metropolis executes in a half-sweep with `accepts` accepted flips, by
    the kind the autotuner picked: (bf16 tensor flops, FP64 flops, what).
      submatrix (tc_flush 2, or 3 split per block): per 32-site block with m accepts, Gamma's m x m products and the
        rank-1 updates of the block in FP64, T = Gamma R_A (N x m x m) and the flush
        G -= G0(:, I_A) T (N x N x m) as 6 x 7-bit slice products (21 pairs);
      delayed (tc_flush 0 / 1): the corrected diagonal and the u, w vectors per accept in FP64
        (about 4 N k), the flush G -= U V^T (N x N x k) in FP64 or as 21 slice pairs."""
    N, Lt = d.L ** 2, d.Lt
    S = 1 if d.model == 1 else 2
    nb = -(-N // 32)
    p_acc = accepts / (N * Lt) if N * Lt else 0.0
    m2 = block_accepts_sq(p_acc) * nb * Lt  # sum over blocks of m^2 in the half-sweep
    m3 = (32 * p_acc) ** 3 * nb * Lt  # and of m^3 (mean-field)
    if tc_flush in (2, 3):
        bf16 = S * 21 * 2 * (N * N * accepts + N * m2)
        fp64 = S * (accepts * 2 * 32 * 32 / 3 + 2 * m2 * 32 + 2 * m3 / 3)
        what = ("submatrix updates: flush and T as 21 bf16 slice pairs of 2 N^2 m + 2 N m^2 per block; "
                "FP64 block updates and Gamma")
    elif tc_flush == 1:
        bf16 = S * 21 * 2 * N * N * accepts
        fp64 = S * accepts * 4 * N * max(kd, 1)
        what = "delayed updates: flush as 21 bf16 slice pairs of 2 N^2 per accept; FP64 vectors"
    else:
        bf16 = 0.0
        fp64 = S * (2 * N * N * accepts + accepts * 4 * N * max(kd, 1))
        what = "delayed updates: FP64 flush 2 N^2 per accept and FP64 vectors"
    return bf16, fp64, what


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
        # an observable the walkers share to rounding (the filling at half filling, the sign of a
        # sign-free model) has no statistical error to compare against
        spread = se > 1e-12 * max(1.0, float(abs(vf[:, k]).max()))
        out[name] = {"abs_diff": d, "fp64_stderr": se, "in_stderr": d / se if spread else None}
    return out


def dg_series(mixed_traces, fp64_traces, descs, same):
    """Max |dG| over the sampled walkers at each stabilization of a forward half-sweep, in
    order (walkers with fewer stabilizations stop early)."""
    import numpy as np

    ns_max = max(-(-d.Lt // d.pace) for d in descs)
    out = []
    for i in range(ns_max):
        vals = [float(np.abs(mixed_traces[w][i] - fp64_traces[w][i]).max())
                for w, d in enumerate(descs) if same[w] and i < -(-d.Lt // d.pace)]
        if vals:
            out.append(max(vals))
    return out


def sample_walkers(descs, wl):
    """The walkers of the accuracy sample: 8 for a uniform batch of small walkers, 2 of the
    large ones, one per side of the uneven batch."""
    if wl.get("uneven"):
        per = len(descs) // 4
        return [descs[k * per] for k in range(4)]
    return descs[: (2 if wl["L"] >= 24 else 8)]


def fp64_comparison(args, dq, wl, stream, step_of):
    """The FP64 path on the same configuration (throughput), the plain single-walker FP64
    path, and |dG| of the mixed path against FP64 at every stabilization of one 0->beta
    half-sweep on the same fields and uniforms (a sample of walkers)."""
    import torch

    def timed_rate(descs, steps):
        b = dq.Batch(descs, rng=dq.RNG_PHILOX, precision=dq.FP64)
        b.set_stream(stream.cuda_stream)
        for w in range(len(descs)):
            b.fields_random(w)
        b.init_greens()
        step = step_of(b)
        step(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(steps):
            step(k)
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
    sub = sample_walkers(descs, wl)
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
    series = dg_series(traces[0], traces[1], sub, same)
    try:
        dev = observable_deviation(obs[0], obs[1], dq.OBS_NAMES, dq.write_bin)
        worst = max((v["in_stderr"] for v in dev.values() if v["in_stderr"] is not None), default=None)
    except Exception as e:  # the throughput line must not depend on this report
        dev, worst = {"unavailable": f"{type(e).__name__}: {e}"}, None
    return {"fp64_batch_value": fp64_value, "fp64_batch_ms_per_step": fp64_ms,
            "fp64_single_walker_value": single_value, "fp64_single_walker_ms_per_step": single_ms,
            "max_abs_dG": max(series) if series else None,
            "dG_per_stabilization": series,
            "dG_sample": f"{len(sub)} walkers, every stabilization of one 0->beta half-sweep (the list: max over "
                         f"the walkers at each stabilization, in order), same fields and Philox uniforms",
            "walkers_with_identical_decisions": int(sum(same)),
            "observables_vs_fp64": dev, "max_observable_dev_in_stderr": worst}


def make_step(wl):
    """The step of a workload on a batch: one half-sweep with equal-time measurement,
    alternating 0->beta and beta->0; or, with taus, one measured forth-and-back pair with the
    dynamic half-sweep."""
    taus = list(wl.get("taus") or ())

    def step_of(b):
        if taus:
            def step(k):
                b.sweep_dynamic(taus)
                b.sweep_beta_to_0(measure=True)
        else:
            def step(k):
                if k % 2 == 0:
                    b.sweep_0_to_beta(measure=True)
                else:
                    b.sweep_beta_to_0(measure=True)
        return step

    return step_of


def per_side_rates(args, dq, wl, stream, step_of):
    """Each side of the uneven batch alone (its 64 walkers as one batch): updates/s and the
    autotuner's pick."""
    import torch

    out = {}
    descs = _descs(dq, wl)
    for L in sorted({d.L for d in descs}):
        sub = [d for d in descs if d.L == L]
        b = dq.Batch(sub, rng=dq.RNG_PHILOX, precision=dq.MIXED if wl.get("precision") == "mixed" else dq.FP64)
        b.set_stream(stream.cuda_stream)
        for w in range(len(sub)):
            b.fields_random(w)
        b.init_greens()
        step = step_of(b)
        for k in range(2):
            step(k)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = max(2, min(args.steps, 6))
        e0.record(stream)
        for k in range(n):
            step(k)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / n
        t = b.tuning()
        out[str(L)] = {"walkers": len(sub), "N": L * L, "updates_per_s": b.updates_per_half_sweep() / (ms * 1e-3),
                       "ms_per_step": ms, "tuner_kd": t["kd"], "tuner_flush": t["tc_flush"]}
        b.close()
    return out


def run_gpu(args, wl, rank, world):
    import numpy as np
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
    mixed = wl.get("precision") == "mixed"
    prec = dq.MIXED if mixed else dq.FP64
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
    step_of = make_step(wl)
    step = step_of(batch)

    for k in range(args.warmup):
        step(k)
    acc0 = np.array([batch.accept_count(w) for w in range(len(descs))], dtype=np.float64)
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
    acc1 = np.array([batch.accept_count(w) for w in range(len(descs))], dtype=np.float64)
    launches = batch.launch_count() - launches0
    # per-kernel-class CUDA-event times: the same number of steps replayed again as profiled
    # graphs (event nodes around each class, one branch), after the timed region
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
    # updating half-sweeps per step: every step of the alternating workloads, the backward
    # half of each pair of the dynamic one
    acc_w = (acc1 - acc0) / args.steps  # accepts per walker per step
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    bf16_peak = peaks.get("bf16_tflops_sustained") or 1700.0
    bf16_src = ("MEASURED_PEAKS.json bf16_tflops_sustained (the class runs inside a long step)"
                if "bf16_tflops_sustained" in peaks else "fallback 1.7 PFLOP/s sustained bf16")
    fp64_src = "FP64 FMA probe measured in this run (dqmc_microbench_fp64); MEASURED_PEAKS.json holds no FP64 figure"
    steps = args.steps
    dyn = bool(wl.get("taus"))
    model = {}  # class -> (bound, algorithmic flops in the profiled steps, peak TFLOP/s, what is counted)
    extra = {}
    if mixed:
        prod = push = greens = bf_met = fp_met = ref_rank1 = dynp = dstab = 0.0
        met_what = ""
        for d, a in zip(descs, acc_w):
            N, S = d.L ** 2, (1 if d.model == 1 else 2)
            ns = -(-d.Lt // d.pace)
            pairs = slice_pairs(wrap_slices(N))
            # forward: 2 wraps + chain; backward: chain + 2 wraps: 3 products per slice of a
            # half-sweep; a step of the dynamic workload is two half-sweeps, whose dynamic one
            # adds the G(t,0) and G(0,t) steps (2 products per slice, class "dynamic")
            prod += steps * S * d.Lt * 3 * pairs * 2 * N ** 3 * (2 if dyn else 1)
            if dyn:
                dynp += steps * S * d.Lt * 2 * pairs * 2 * N ** 3
            if N >= 128:
                pf, gf = stab_tensor_flops(N)
                sp = slice_pairs(8 if N <= 256 else 9)
                push += steps * S * ns * pf * sp
                greens += steps * S * ns * gf * sp
                if dyn:  # the dynamic half-sweep's assembly with its second right-hand side and outputs
                    dstab += steps * S * ns * (gf + stab_rhs_flops(N) + 2 * 2 * N ** 3) * sp
            b_, f_, met_what = metropolis_work(d, a, tuning["tc_flush"], tuning["kd"])
            bf_met += steps * b_
            fp_met += steps * f_
            ref_rank1 += steps * S * a * 2 * N * N
        model["product"] = ("tensor", prod, bf16_peak,
                            "BF16 flops of the exact-slice wrap and B-chain products: 3 per slice x slice pairs "
                            "(28 for N <= 256, 36 above) x 2N^3")
        if dstab > 0:
            model["dynamic_stab"] = ("tensor", dstab, bf16_peak,
                                     "BF16 flops of the dynamic half-sweep's blocked-QR Green's assembly with the "
                                     "second right-hand side and the G(t,0), G(0,t) products (45 slice pairs above "
                                     "N = 256, 36 below)")
        if dyn:
            model["dynamic"] = ("tensor", dynp, bf16_peak,
                                "BF16 flops of the G(t,0), G(0,t) steps of the dynamic half-sweep (2 products "
                                "per slice x slice pairs x 2N^3); its G(k,tau) measurement runs in the same class")
        if push > 0:
            # the dynamic half-sweep's push and equal-time assembly run in the same classes
            # (its assembly for tensor-core walkers is timed under dynamic_stab): counted as
            # many blocked-QR products again in push, not in greens
            model["push"] = ("tensor", push * (2 if dyn else 1), bf16_peak,
                             "BF16 flops of the blocked-QR products (36 slice pairs, 45 for N > 256)")
            model["greens"] = ("tensor", greens, bf16_peak,
                               "BF16 flops of the Green's-assembly products (36 slice pairs, 45 for N > 256)")
        model["metropolis"] = ("tensor", bf_met, bf16_peak, met_what)
        extra["metropolis"] = {"fp64_flops_executed_tflops": None, "fp64_frac": None,
                               "reference_rank1_equivalent_tflops": None,
                               "note": "the reference's rank-1 FP64 flops (2 N^2 per accepted flip and spin) over "
                                       "this class's time: an algorithm-equivalent rate, not a roofline"}
        extra["_fp64_met"] = fp_met
        extra["_ref_rank1"] = ref_rank1
    else:
        tot = {"segment": 0.0, "push": 0.0, "greens": 0.0}
        for d, a in zip(descs, acc_w):
            fm = flops_model(d, a)
            for k in tot:
                tot[k] += steps * fm[k]
        for k in ("segment", "push", "greens"):
            model[k] = ("fp64", tot[k], fp64_peak / 1e3,
                        "FP64 flops of the class (flops_model: wraps, chain products, Green's assembly)")
    timed_classes = [k for k in model if prof.get(k, (0, 0))[1] > 0 and model[k][1] > 0]
    dom = max(timed_classes, key=lambda k: prof[k][0]) if timed_classes else max(prof, key=lambda k: prof[k][0])
    classes = {k: {"bound": v[0], "achieved_tflops": v[1] / (prof[k][0] * 1e-3) / 1e12,
                   "frac": v[1] / (prof[k][0] * 1e-3) / 1e12 / v[2], "counted": v[3]}
               for k, v in model.items() if prof.get(k, (0, 0))[0] > 0}
    if "metropolis" in classes and "_fp64_met" in extra:
        t_s = prof["metropolis"][0] * 1e-3
        m = extra["metropolis"]
        m["fp64_flops_executed_tflops"] = extra["_fp64_met"] / t_s / 1e12
        m["fp64_frac"] = m["fp64_flops_executed_tflops"] / (fp64_peak / 1e3)
        m["reference_rank1_equivalent_tflops"] = extra["_ref_rank1"] / t_s / 1e12
        classes["metropolis"].update(m)
    if dom in model:
        bound, flops, peak, what = model[dom]
    else:
        bound, flops, peak, what = ("tensor" if mixed else "fp64"), None, None, "no flop model for this class"
    dom_ms, dom_n = prof[dom]
    achieved = flops / (dom_ms * 1e-3) / 1e12 if flops else None
    # the profiled replay runs one branch, so each of its launches covers every walker
    traffic, traffic_kernel, traffic_src = ncu_traffic(wl, dom, len(descs))
    roofline = {"bound": bound, "kernel": f"{dom} kernel class", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "traffic_kernel": traffic_kernel, "traffic_source": traffic_src,
                "peak_source": bf16_src if bound == "tensor" else fp64_src, "counted": what,
                "avg_launch_ms": dom_ms / max(dom_n, 1),
                "kernel_share": {k: prof[k][0] / prof_total for k in prof if prof[k][1] > 0},
                "profiled_ms_per_step": prof_total / args.steps,
                "classes": classes}
    if not mixed:
        nominal = sum(steps * flops_model(d, a)["nominal_F"] for d, a in zip(descs, acc_w))
        roofline["sweep_nominal_F_tflops"] = nominal / (ms * 1e-3) / 1e12

    # ---- e2e: reference RNG on the host, copies in and out every step
    e2e = None
    if rank == 0 or world > 1:
        eb = dq.Batch(descs, rng=dq.RNG_MINSTD, precision=prec)
        eb.set_stream(stream.cuda_stream)
        for w in range(len(descs)):
            eb.fields_random(w)
        eb.init_greens()
        estep = step_of(eb)
        for k in range(max(1, min(args.warmup, 3))):
            estep(k)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        ek = max(2, min(args.steps, 10))
        d2h = 0
        for k in range(ek):
            estep(k)
            sums, counts = eb.observables_all()
            d2h = int(sums.nbytes + counts.nbytes)
            if dyn:
                for w in range(len(descs)):
                    ds, dc = eb.dynamic(w)
                d2h += len(descs) * int(ds.nbytes + dc.nbytes)
        el = time.perf_counter() - t0
        barrier()
        e2e = {"value": world * upd * ek / el, "unit": "updates/s",
               "h2d_bytes_per_step": 8 * upd, "d2h_bytes_per_step": d2h,
               "steps": ek, "rng": "host minstd_rand0 (reference stream)"}
        eb.close()
    cmp = None
    side = None
    if mixed and rank == 0 and world == 1 and not args.no_compare:
        cmp = fp64_comparison(args, dq, wl, stream, step_of)
        if wl.get("uneven"):
            side = per_side_rates(args, dq, wl, stream, step_of)
    return dict(value=value, ms=ms, roofline=roofline, e2e=e2e, clocks=clk, launches=launches, status=status,
                tuning=tuning, fp64=cmp, per_side=side,
                accept_rate=float(acc_w.sum() / max(upd, 1)), fp64_peak=fp64_peak)


def workload_config(name, wl, gpus):
    if wl.get("uneven"):
        c = {"workload": name, "walkers_per_gpu": wl["walkers"], "model": "repulsive", "L": [6, 8, 10, 12],
             "walkers_per_side": wl["walkers"] // 4, "N": [36, 64, 100, 144],
             "U": "per walker, 2 + 4u, u canonical from std::mt19937_64(7)",
             "beta": "per walker, (4, 6, 8)[floor(3u')] from the same engine", "dtau": 0.05, "mu": 0.0,
             "pace": wl["pace"], "expK": "dense"}
    else:
        c = {"workload": name, "walkers_per_gpu": wl["walkers"],
             "model": "repulsive" if wl["model"] == 0 else "attractive",
             "L": wl["L"], "N": wl["L"] ** 2, "U": wl["U"], "mu": wl["mu"], "beta": wl["beta"], "Lt": wl["Lt"],
             "pace": wl["pace"], "expK": "checkerboard" if wl["checkerboard"] else "dense"}
    c["precision"] = wl.get("precision", "fp64")
    if wl.get("taus"):
        c["measure"] = ("one step = one measured forth-and-back pair: dynamic 0->beta half-sweep with G(k,tau) and "
                        "the dynamic observables at tau = " + ",".join(str(t) for t in wl["taus"]) +
                        ", then the updating beta->0 half-sweep with equal-time measurement; updates counted "
                        "for the updating half-sweep only")
    else:
        c["measure"] = "equal-time, fused; one step = one half-sweep"
    c["parallelism"] = f"replicas x{gpus}"
    c["l2"] = l2_note(wl)
    return c


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
    config = workload_config(args.workload, wl, args.gpus)

    if args.impl == "reference":
        if rank != 0:
            return
        # the reference arm times what it runs: `steps` steps per host core (fewer if the
        # budget runs out first; the line then says how many), one walker per core
        cb = cpu_baseline(wl, budget_s=max(30.0, args.cpu_budget * 5), steps=max(1, args.steps))
        line = {"metric": METRIC, "value": cb["value"], "unit": "updates/s", "n_gpus": args.gpus,
                "steps": cb["steps"], "warmup": 1, "ms_per_step": cb["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded +/-1 fields)", "config": dict(config, timed_walkers=cb["cores"],
                                                                        timed_what="one walker per host core; "
                                                                        "ms_per_step is one core's time per step"),
                "impl": "reference",
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
    if r["per_side"]:
        line["per_side"] = r["per_side"]
    if r["fp64"]:
        c = r["fp64"]
        line["vs_fp64"] = dict(c, ratio_vs_fp64_batch=r["value"] / c["fp64_batch_value"],
                               ratio_vs_fp64_single_walker=r["value"] / c["fp64_single_walker_value"])
    print(json.dumps(line))


if __name__ == "__main__":
    main()
