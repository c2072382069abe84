"""The reference-style driver (python -m dqmc_gb300.run) end to end on the GPU, and
the HBM path at shared-memory sizes (the dynamic half-sweep needs it there)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIG = """
[Model]
    type = "RepulsiveHubbard"
    [Model.Params]
    hopping_t = 1.0
    onsite_u = 4.0
    chemical_potential = 0.0
[Lattice]
    type = "Square"
    cell = [ 4, 4 ]
    momentum = "MPoint"
[MonteCarlo]
    beta = 1.0
    time_size = 10
    stabilization_pace = 5
[Measure]
    sweeps_warmup = 4
    bin_num = 4
    bin_size = 4
    sweeps_between_bins = 2
    observables = [ "all" ]
"""


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build()
    import dqmc_gb300

    return dqmc_gb300


def test_hbm_path_equals_shared_memory_path(dq):
    """N = 16 walkers on the HBM path (hbm option) against the shared-memory path:
    identical decisions and G within 1e-10 after full sweeps with measurements."""
    descs = [dq.WalkerDesc(model=m, L=4, U=4.0, mu=-0.3 * m, beta=1.0, Lt=10, pace=5, seed=40 + m) for m in (0, 1)]
    out = []
    for hbm in (False, True):
        b = dq.Batch(descs, rng=dq.RNG_MINSTD, hbm=hbm)
        for w in range(2):
            b.fields_random(w)
        b.init_greens()
        for _ in range(2):
            b.sweep_0_to_beta(measure=True)
            b.sweep_beta_to_0(measure=True)
        out.append(([b.fields(w) for w in range(2)], [b.green(w, s) for w in range(2) for s in (0, 1)],
                    b.observables_all()[0]))
        b.close()
    (f0, g0, o0), (f1, g1, o1) = out
    for w in range(2):
        np.testing.assert_array_equal(f0[w], f1[w])
    for a, c in zip(g0, g1):
        assert abs(a - c).max() < 1e-10
    np.testing.assert_allclose(o0, o1, rtol=1e-10, atol=1e-12)


def test_driver_runs_a_reference_config(dq, tmp_path):
    from dqmc_gb300 import io as dio
    from dqmc_gb300.run import run

    cfg = dio.parse_config(CONFIG)
    log = tmp_path / "log.txt"
    with open(log, "w") as fh:
        res = run(cfg, str(tmp_path), walkers=2, seed=7, log=fh)
    for name in ("fields.out", "kstars.out", "tgrids.out", "swave.out", "swave.bins.out", "dos.out",
                 "dos.bins.out", "greens.out", "greens.bins.out", "dss.out", "dss.bins.out"):
        assert os.path.getsize(tmp_path / name) > 0, name
    dos = open(tmp_path / "dos.out").read().splitlines()
    assert int(dos[0]) == 10 and len(dos) == 11
    bins = open(tmp_path / "dos.bins.out").read().splitlines()
    assert bins[0].split() == ["4", "10"]  # 2 walkers x ceil(4 / 2) bins, 10 tau
    greens = open(tmp_path / "greens.out").read().splitlines()
    assert greens[0].split() == ["6", "10"]  # every k star of the 4 x 4 lattice, 10 tau
    lt, n, _ = dio.parse_fields(open(tmp_path / "fields.out").read())
    assert (lt, n) == (10, 16)
    # half filling without a sign problem: <n> = 1, sign 1; D(0) = tr G / N near 1/2
    assert res["equaltime_sign"][0] == pytest.approx(1.0) and res["dynamic_sign"][0] == pytest.approx(1.0)
    assert abs(res["filling_number"][0] - 1.0) < 0.05
    d0 = float(dos[1].split()[1])
    assert abs(d0 - 0.5) < 0.05
    assert np.isfinite(res["superfluid_stiffness"][0])
    text = open(log).read()
    assert "Filling number" in text and "Superfluid stiffness" in text


def test_device_binning_equals_host_binning(dq):
    """dqmc_measure_bins (binning by a kernel, one copy at the end) against the host loop
    with dqmc_get_observables_all + write_bin on an identical batch (Philox uniforms)."""
    descs = [dq.WalkerDesc(model=m % 2, L=4, U=4.0, mu=-0.2 * (m % 2), beta=1.0, Lt=10, pace=5, seed=60 + m)
             for m in range(3)]
    nbins, size, between = 3, 4, 2
    a = dq.Batch(descs, rng=dq.RNG_PHILOX)
    b = dq.Batch(descs, rng=dq.RNG_PHILOX)
    for bb in (a, b):
        for w in range(3):
            bb.fields_random(w)
        bb.init_greens()
    dev = a.measure_bins(nbins, size, between)
    host = np.zeros_like(dev)
    b.clear_observables()
    for k in range(nbins):
        for _ in range(size // 2):
            b.sweep_0_to_beta(measure=True)
            b.sweep_beta_to_0(measure=True)
        sums, counts = b.observables_all()
        for w in range(3):
            host[w, k] = dq.write_bin(sums[w], counts[w])
        b.clear_observables()
        for _ in range(between // 2):
            b.sweep_0_to_beta()
            b.sweep_beta_to_0()
    np.testing.assert_allclose(dev, host, rtol=1e-14, atol=0)
    for w in range(3):
        np.testing.assert_array_equal(a.fields(w), b.fields(w))
