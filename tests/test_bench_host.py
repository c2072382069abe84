"""bench.py's host logic, without a GPU: the flop model of the roofline (the per-walker
work of a half-sweep, dqmc_walker.cpp:246-412 counted as the reference executes it), the
ncu traffic attached to the dominant class, and the reference arm's JSON line (the CPU
restatement of the reference, timed on this machine's cores for a few seconds)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, ROOT)
    import bench as b

    return b


def test_flop_model_counts_the_reference_work(bench):
    wl = dict(bench.WORKLOADS["fp64_single_4x4_dense"])  # N = 16, Lt = 80, pace 10, repulsive
    N, Lt, S = 16, 80, 2
    A = 300.0  # accepted flips per half-sweep
    fm = bench.flops_model(wl, A)
    W, C = 4 * N ** 3 + 2 * N * N, 2 * N ** 3 + N * N  # dense wrap and B-chain step
    assert fm["segment"] == S * Lt * (W + C) + S * A * 2 * N * N
    ns = Lt // 10
    assert fm["push"] == pytest.approx(S * ns * (8 / 3 + 1) * N ** 3)
    assert fm["nominal_F"] == S * Lt * (W + C) + S * A * 2 * N * N + S * ns * 33 * N ** 3
    cb = bench.flops_model(dict(bench.WORKLOADS["fp64_batch_8x8_checkerboard"]), 0.0)
    assert cb["segment"] == 2 * 160 * (34 + 17) * 64 * 64  # checkerboard passes, no flips


def test_blocked_qr_products_flops(bench):
    """Each panel of the blocked QR costs its trailing update and the Q formation; the counts
    grow like N^3 and exceed the plain 2N^3 products they include."""
    p1, g1 = bench.stab_tensor_flops(128)
    p2, g2 = bench.stab_tensor_flops(256)
    assert p1 > 2 * 128 ** 3 and g1 > 6 * 128 ** 3
    assert 6 < p2 / p1 < 10 and 6 < g2 / g1 < 10


def test_traffic_of_the_dominant_class(bench):
    wl = dict(bench.WORKLOADS["mixed_batch_16x16_attractive"])
    t, kern, src = bench.ncu_traffic(wl, "metropolis", 128)
    assert kern == "metropolis_sub_kernel" and t == 4379392 * 16  # the 8-walker capture, scaled to 128
    assert "8-walker" in src and "128 walkers" in src
    assert bench.ncu_traffic(wl, "product", 8)[0] == 8307200
    for w, cls in ((bench.WORKLOADS["fp64_batch_8x8_checkerboard"], "segment"), (wl, "greens")):
        t, kern, src = bench.ncu_traffic(dict(w), cls, 64)
        assert t is None and kern is None and src


@pytest.mark.timeout(600)
def test_reference_arm_prints_the_contract_line():
    """--impl reference: one JSON line with impl, cpu_baseline (kind, cores, sample, value equal
    to the line's) and e2e with zero copies, on the metric and unit of the GPU arm."""
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "fp64_single_4x4_dense", "--steps", "1", "--warmup", "0",
                          "--cpu-budget", "2"], capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "updates/s" and d["higher_is_better"] is True
    assert d["metric"].startswith("HS-field updates/s")
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] > 0 and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == "fp64_single_4x4_dense"
    # the line states what it timed: steps per core and one core's time per step, which fit the run
    assert d["steps"] == 1 and d["config"]["timed_walkers"] == cb["cores"]
    assert 0 < d["steps"] * d["ms_per_step"] < 600e3


def test_slice_pair_counts(bench):
    """Wraps and B-chain: 7 slices (28 pairs) up to N = 256, 8 slices (36 pairs) above, the
    configurations of ozaki::cfg_for_k."""
    assert bench.wrap_slices(256) == 7 and bench.wrap_slices(257) == 8
    assert bench.slice_pairs(7) == 28 and bench.slice_pairs(8) == 36 and bench.slice_pairs(6) == 21


def test_metropolis_work_by_update_kind(bench):
    """The Metropolis class is counted by the work it executes: the submatrix flush's bf16
    slice products (21 pairs of 2 N^2 per accept plus the m^2 terms of T), its small FP64 part,
    and the FP64 flush of the delayed kernel."""
    sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
    import dqmc_gb300 as dq

    d = dq.WalkerDesc(model=1, L=16, U=4.0, mu=-0.5, beta=10.0, Lt=100, pace=8)
    N, A = 256, 0.6 * 256 * 100
    bf, fp, what = bench.metropolis_work(d, A, 2, 32)
    assert bf >= 21 * 2 * N * N * A and bf < 1.2 * 21 * 2 * N * N * A
    assert 0 < fp < 0.05 * 2 * N * N * A and "submatrix" in what
    bf0, fp0, _ = bench.metropolis_work(d, A, 0, 16)
    assert bf0 == 0 and fp0 >= 2 * N * N * A
    bf1, _, _ = bench.metropolis_work(d, A, 1, 32)
    assert bf1 == 21 * 2 * N * N * A


def test_uneven_workload_walkers(bench):
    """The uneven batch: 64 walkers of each side 6, 8, 10, 12, Lt from beta in {4, 6, 8} at
    dtau = 0.05, |U| in [2, 6); its per-side CPU samples cover every side."""
    sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
    import dqmc_gb300 as dq

    wl = bench.WORKLOADS["mixed_uneven_6_to_12"]
    descs = bench._descs(dq, wl)
    assert len(descs) == 256
    assert {L: sum(1 for d in descs if d.L == L) for L in (6, 8, 10, 12)} == {6: 64, 8: 64, 10: 64, 12: 64}
    assert {d.Lt for d in descs} == {80, 120, 160} and all(2 <= d.U < 6 for d in descs)
    assert all(d.Lt == round(d.beta / 0.05) and d.pace == 10 for d in descs)
    samples, _ = bench._cpu_samples(wl, 16)
    assert sorted({p["L"] for p, _ in samples}) == [6, 8, 10, 12]
    assert bench.working_set_bytes(wl) > bench.L2_BYTES


def test_dg_series_per_stabilization(bench):
    """max |dG| over the sampled walkers at each stabilization, in order; walkers whose
    decisions differ are left out."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
    import dqmc_gb300 as dq

    descs = [dq.WalkerDesc(L=4, Lt=20, pace=10), dq.WalkerDesc(L=4, Lt=30, pace=10)]
    z = [np.zeros((3, 2, 16, 16)), np.zeros((3, 2, 16, 16))]
    m = [a.copy() for a in z]
    m[0][0] += 1e-9
    m[1][2] += 3e-8
    m[1][1] += 2e-9
    assert bench.dg_series(m, z, descs, [True, True]) == pytest.approx([1e-9, 2e-9, 3e-8])
    assert bench.dg_series(m, z, descs, [True, False]) == pytest.approx([1e-9, 0.0])


def test_l2_note_follows_the_working_set(bench):
    """The batches' working sets exceed L2 (no flush needed); the single 4x4 walker fits and
    says so."""
    big = bench.WORKLOADS["mixed_batch_16x16_attractive"]
    # per walker: G 2N^2, chain N^2, stacks 2 x 13 levels x (2N^2 + N) doubles (N = 256, S = 1)
    assert bench.working_set_bytes(big) == 128 * 8 * (2 * 65536 + 65536 + 2 * 13 * (2 * 65536 + 256))
    assert bench.l2_note(big).startswith("no flush: the per-GPU working set")
    assert bench.working_set_bytes(bench.WORKLOADS["fp64_batch_8x8_checkerboard"]) > bench.L2_BYTES
    assert "fits in L2" in bench.l2_note(bench.WORKLOADS["fp64_single_4x4_dense"])


def test_observable_deviation_in_units_of_the_stderr(bench):
    """Each observable's mixed-vs-FP64 difference of walker means over the FP64 standard
    error; an observable with no spread (the sign of a sign-free model) reports None."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
    import dqmc_gb300 as dq

    rng = np.random.default_rng(3)
    n, k = 8, dq.NUM_OBS
    counts = np.full((n, k), 100, dtype=np.int64)
    sums_f = rng.normal(1.0, 0.1, (n, k)) * 100
    sums_f[:, -1] = 100.0  # sign = +1 in every walker
    sums_m = sums_f.copy()
    sums_m[:, 2] += 100 * 1e-3  # shift the kinetic energy of every walker by 1e-3
    dev = bench.observable_deviation((sums_m, counts), (sums_f, counts), dq.OBS_NAMES, dq.write_bin)
    vf = sums_f[:, 2] / 100
    se = vf.std(ddof=1) / np.sqrt(n)
    assert dev["kinetic_energy"]["abs_diff"] == pytest.approx(1e-3)
    assert dev["kinetic_energy"]["in_stderr"] == pytest.approx(1e-3 / se)
    assert dev["filling_number"]["abs_diff"] == 0.0 and dev["filling_number"]["in_stderr"] == 0.0
    assert dev["equaltime_sign"]["in_stderr"] is None
    json.dumps(dev)
