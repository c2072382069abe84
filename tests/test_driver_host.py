"""The driver's host logic (dqmc_gb300.run) on the CPU with a stand-in batch: bin
counts per walker, the normalisation of MeasureHandler::normalize_stats for the
equal-time and dynamic observables, pooling and the files written.  The device
path itself is covered by tests/test_gpu_driver.py."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))

import dqmc_gb300 as dq  # noqa: E402  (the ctypes library is only loaded on first use)
from dqmc_gb300 import io as dio  # noqa: E402
from dqmc_gb300 import run as drv  # noqa: E402

SIGN = -0.5  # a constant walker sign: every normalised value is independent of it


class FakeBatch:
    """Answers like dqmc_gb300.Batch for walkers whose every measurement gives the
    same value: equal-time observable k of walker w = 0.1 (k + 1) + w, dynamic
    G(k,tau) = k + tau / 100, D(tau) = 1 + tau, chi(tau) = 2 tau, stiffness term = 0.01."""
    created = []

    def __init__(self, descs, rng=None, precision=None, hbm=False):
        self.descs, self.hbm = list(descs), hbm
        self.nw, self.lt, self.N = len(self.descs), self.descs[0].Lt, self.descs[0].N
        self.half = {"fwd": 0, "bwd": 0, "dyn": 0}
        self.clear_observables()
        self.clear_dynamic()
        FakeBatch.created.append(self)

    def fields_random(self, w): pass
    def set_fields(self, w, f): self.f = f
    def init_greens(self): pass
    def close(self): pass
    def config_sign(self, w): return SIGN
    def wrap_error(self, w): return 1e-9 * (w + 1)
    def fields(self, w): return np.ones((self.lt, self.N), dtype=np.int8)

    def clear_observables(self):
        self.ecount = 0

    def clear_dynamic(self):
        self.dcount = 0

    def sweep_0_to_beta(self, measure=False):
        self.half["fwd"] += 1
        self.ecount += measure

    def sweep_beta_to_0(self, measure=False):
        self.half["bwd"] += 1
        self.ecount += measure

    def sweep_dynamic(self, taus):
        assert taus == list(range(self.lt))
        self.half["dyn"] += 1
        self.dcount += 1

    def observables_all(self):
        val = np.array([[0.1 * (k + 1) + w for k in range(dq.NUM_OBS)] for w in range(self.nw)])
        cnt = np.full((self.nw, dq.NUM_OBS), self.ecount * self.lt, dtype=np.int64)
        sums = cnt * val * SIGN
        sums[:, -1] = cnt[:, -1] * SIGN
        return sums, cnt

    def measure_bins(self, nbins, size, between):
        out = np.zeros((self.nw, nbins, dq.NUM_OBS))
        for k in range(nbins):
            self.clear_observables()
            for _ in range(size // 2):
                self.sweep_0_to_beta(True)
                self.sweep_beta_to_0(True)
            s, c = self.observables_all()
            out[:, k] = [dq.write_bin(s[w], c[w]) for w in range(self.nw)]
            for _ in range(between // 2):
                self.sweep_0_to_beta()
                self.sweep_beta_to_0()
        return out

    def _c(self):
        return np.full(self.lt, self.dcount, dtype=np.int64)

    def dynamic(self, w):
        return self.dcount * SIGN * (np.arange(self.lt) / 100.0), self._c()

    def dynamic_obs(self, w):
        t = np.arange(self.lt)
        return self.dcount * SIGN * (1.0 + t), self.dcount * SIGN * 2.0 * t, np.full(self.lt, self.dcount * SIGN * 0.01)

    def dynamic_greens_k(self, w, momenta):
        return np.array([[self.dcount * SIGN * (k + tau / 100.0) for tau in range(self.lt)]
                         for k in range(len(momenta))])


CONFIG = """
[Model]
    type = "RepulsiveHubbard"
[Lattice]
    cell = [ 4, 4 ]
    momentum = "MPoint"
    momentum_list = "DeltaLine"
[MonteCarlo]
    beta = 1.0
    time_size = 6
    stabilization_pace = 3
[Measure]
    sweeps_warmup = 4
    bin_num = 5
    bin_size = 4
    sweeps_between_bins = 2
    observables = [ %s ]
"""


@pytest.fixture
def fake(monkeypatch):
    FakeBatch.created.clear()
    monkeypatch.setattr(dq, "Batch", FakeBatch)
    return FakeBatch


def test_equaltime_run(fake, tmp_path):
    cfg = dio.parse_config(CONFIG % '"filling_number", "s_wave_pairing_corr"')
    with open(tmp_path / "log", "w") as log:
        res = drv.run(cfg, str(tmp_path), walkers=2, log=log)
    b = fake.created[0]
    assert not b.hbm  # equal-time only: walkers keep the shared-memory path
    # 2 warm-up pairs, ceil(5 / 2) = 3 bins of 2 measured pairs and 1 pair between
    assert b.half["fwd"] == b.half["bwd"] == 2 + 3 * 2 + 3
    # pooled over 2 walkers x 3 bins: filling (k = 0) = mean of 0.1 and 1.1
    assert res["filling_number"][0] == pytest.approx(0.6)
    assert res["equaltime_sign"] == (pytest.approx(0.5), pytest.approx(0.0))
    swave = open(tmp_path / "swave.out").read()
    assert swave.startswith(dio._f(0.8 + 0.5))
    assert open(tmp_path / "swave.bins.out").read().splitlines()[0] == dio._d(6)
    assert not os.path.exists(tmp_path / "dos.out")
    text = open(tmp_path / "log").read()
    assert "Filling number" in text
    # dqmc_main's layout: start-up lines, the parameter block, the ending info with the
    # largest wrap error over the walkers, the signs, a blank line, the observables
    assert text.startswith(">> Configurations of the bosonic fields set to random.\n\n>> Initialization finished.")
    assert "   Model: Repulsive Hubbard\n" in text and dio._param("Number of bins", "6") in text
    assert ">> Maximum of the wrapping error: 2.00000e-09\n" in text
    signs, rest = text.split(">> Maximum of the wrapping error: 2.00000e-09\n\n")[1].split("\n\n", 1)
    assert signs.strip().startswith("Averaged sign (equal-time)")
    assert rest.index("Filling number") < rest.index("S-wave pairing correlation")


def test_dynamic_run(fake, tmp_path):
    cfg = dio.parse_config(CONFIG % '"all"')
    res = drv.run(cfg, str(tmp_path), walkers=3, log=open(os.devnull, "w"))
    b = fake.created[0]
    assert not b.hbm  # shared-memory walkers run the dynamic half-sweep too
    # ceil(5 / 3) = 2 bins of 2 dynamic + backward pairs; forward half-sweeps only in warm-up and between
    assert b.half["dyn"] == 2 * 2 and b.half["fwd"] == 2 + 2 * 1 and b.half["bwd"] == 2 + 2 * 2 + 2 * 1
    dos = open(tmp_path / "dos.out").read().splitlines()
    assert dos[0] == dio._d(6) and dos[3].startswith(dio._d(2) + dio._f(3.0))
    dss = open(tmp_path / "dss.out").read().splitlines()
    assert dss[2].startswith(dio._d(1) + dio._f(2.0))
    greens = open(tmp_path / "greens.out").read().splitlines()
    assert greens[0] == dio._d(3) + dio._d(6)  # DeltaLine of the 4 x 4 lattice: 3 k stars
    assert greens[-1].startswith(dio._d(2) + dio._d(5) + dio._f(2.05))
    assert res["superfluid_stiffness"][0] == pytest.approx(0.06)  # 6 tau x 0.01
    assert res["dynamic_sign"][0] == pytest.approx(0.5)
    assert open(tmp_path / "greens.bins.out").read().splitlines()[0] == dio._d(6) + dio._d(3) + dio._d(6)


def test_cubic_configuration_runs_cubic_walkers(fake, tmp_path):
    """A cubic configuration (dqmc_initializer.cpp:118-150) gives walkers of the cubic
    lattice with N = L^3, its measured momentum and momentum list from the cubic
    tables, and no superfluid stiffness (dqmc_initializer.cpp:233-237)."""
    cfg = dio.parse_config('[Lattice]\ntype = "Cubic"\ncell = [4, 4, 4]\nmomentum = "XPoint"\n'
                           'momentum_list = "LambdaLine"\n[MonteCarlo]\nbeta = 1.0\ntime_size = 6\n'
                           'stabilization_pace = 3\n[Measure]\nsweeps_warmup = 2\nbin_num = 2\nbin_size = 2\n'
                           'sweeps_between_bins = 0\nobservables = ["all"]\n')
    res = drv.run(cfg, str(tmp_path), walkers=1, log=open(os.devnull, "w"))
    d = fake.created[0].descs[0]
    assert d.lattice == dq.CUBIC and d.N == 64 and fake.created[0].N == 64
    assert d.momentum_index == dio.momentum_index(4, "XPoint", 3)
    assert "superfluid_stiffness" not in res and "filling_number" in res
    greens = open(tmp_path / "greens.out").read().splitlines()
    nline = len(dio.momentum_list_indices(4, "LambdaLine", 3))
    assert greens[0] == dio._d(nline) + dio._d(6)
    assert len(open(tmp_path / "kstars.out").read().splitlines()) == 1 + len(dio.kstars(4, 3))  # count line


def test_reference_command_line_and_fields_resume(fake, tmp_path):
    """dqmc_main's options (-c/--config, -o/--output, -f/--fields, src/dqmc_main.cpp:53-62): the
    run starts from the fields file and writes the final fields back over it
    (src/dqmc_main.cpp:280-283), and the output folder is created."""
    cfg_path = tmp_path / "config.toml"
    cfg_path.write_text(CONFIG % '"filling_number"')
    start = [[-1] * 16 for _ in range(6)]
    fpath = tmp_path / "fields.in"
    fpath.write_text(dio.format_fields(start))
    out = tmp_path / "out" / "run1"
    import contextlib
    import io as sio

    with contextlib.redirect_stdout(sio.StringIO()) as buf:
        assert drv.main(["--config", str(cfg_path), "--output", str(out), "--fields", str(fpath), "--walkers", "2"]) == 0
    b = fake.created[0]
    assert (b.f == -1).all()  # started from the file
    lt, n, f = dio.parse_fields(fpath.read_text())
    assert (lt, n) == (6, 16) and all(v == 1 for row in f for v in row)  # FakeBatch's final fields
    assert not (out / "fields.out").exists() and (out / "kstars.out").exists()
    assert "read from the input config file" in buf.getvalue()
    with contextlib.redirect_stdout(sio.StringIO()):
        assert drv.main(["-c", str(cfg_path), "-o", str(tmp_path / "o2")]) == 0
    assert (tmp_path / "o2" / "fields.out").exists()
    with pytest.raises(SystemExit):
        drv.main(["-o", str(tmp_path / "o3")])  # no configuration
