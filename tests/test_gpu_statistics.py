"""Statistical parity of the GPU path with the reference's shipped run.

The C++ driver (apps/dqmc_run.cpp, written against include/dqmc_gb300.hpp in
the reference's DqmcWalker / MeasureHandler / Dqmc vocabulary) runs the
example configuration of the reference (attractive Hubbard 8x8, U=4, beta=8,
Lt=160, pace 10, dense exp(-dtau K)) warm-started from its fields.out, with
64 walkers in one batch, and every equal-time observable must agree with
example/log.out:44-55 within 4 combined standard errors.
"""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_example_run_matches_reference_log(example_fixture, tmp_path):
    import __graft_entry__ as g

    g.build()
    fields = example_fixture["fields"]
    path = tmp_path / "fields.out"
    with open(path, "w") as f:  # DqmcIO::output_bosonic_fields layout (include/dqmc_io.h:496-506)
        f.write(f"{fields.shape[0]:20d}{fields.shape[1]:20d}\n")
        for t in range(fields.shape[0]):
            for i in range(fields.shape[1]):
                f.write(f"{t:20d}{i:20d}{float(fields[t, i]):20.1f}\n")
    exe = os.path.join(ROOT, "dqmc-framework_gb300", "lib", "dqmc_run")
    args = [exe, "model=attractive", "L=8", "U=4", "beta=8", "Lt=160", "pace=10", "checkerboard=0",
            "walkers=64", "seed=2024", "warmup=20", "bins=4", "binsize=40", "between=0", f"fields={path}",
            "rng=philox"]
    out = subprocess.run(args, check=True, capture_output=True, text=True, timeout=600).stdout
    res = json.loads(out.strip().splitlines()[-1])
    assert res["bins"] == 64 * 4
    assert 1e-12 < res["max_wrap_error"] < 1e-6
    for name, (ref, ref_err) in example_fixture["observables"].items():
        mean, err = res[name]
        sigma = np.hypot(err, ref_err)
        if sigma == 0:
            assert mean == pytest.approx(ref)
        else:
            assert abs(mean - ref) < 4 * sigma, (name, mean, err, ref, ref_err)


def test_example_run_256_chains_autocorrelation_aware(example_fixture):
    """The same configuration with 256 independent chains (walkers), each warm-started from
    fields.out, 20 warm-up half-sweeps and 4 bins of 40 measured half-sweeps with device-side
    binning.  The error of each observable comes from the 256 chain means (independent
    chains, so the autocorrelation of bins within a chain does not shrink it), and every
    equal-time observable must lie within 3 combined standard errors of example/log.out
    (the deviations are printed)."""
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300 as dq

    nw = 256
    descs = [dq.WalkerDesc(model=1, L=8, U=4.0, mu=0.0, beta=8.0, Lt=160, pace=10, seed=3000 + w) for w in range(nw)]
    b = dq.Batch(descs, rng=dq.RNG_PHILOX)
    for w in range(nw):
        b.set_fields(w, example_fixture["fields"])
    b.init_greens()
    for _ in range(10):
        b.sweep_0_to_beta()
        b.sweep_beta_to_0()
    bins = b.measure_bins(4, 40, 0)  # [walker][bin][obs]
    assert all(b.status(w) == 0 for w in range(nw))
    chain = bins.mean(axis=1)  # [walker][obs]
    mean = chain.mean(axis=0)
    err = chain.std(axis=0, ddof=1) / np.sqrt(nw)
    devs = {}
    for k, name in enumerate(dq.OBS_NAMES):
        if name not in example_fixture["observables"]:
            continue
        ref, ref_err = example_fixture["observables"][name]
        sigma = np.hypot(err[k], ref_err)
        if sigma == 0:
            assert mean[k] == pytest.approx(ref)
            continue
        devs[name] = abs(mean[k] - ref) / sigma
    print("MEASURED deviations from example/log.out in combined standard errors:",
          {k: round(v, 2) for k, v in devs.items()})
    for name, d in devs.items():
        assert d < 3.0, (name, d)
