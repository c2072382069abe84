"""The two drivers over the same stand-in library: the Python driver (dqmc_gb300.run, whose
device run is tested on the GPU by tests/test_gpu_driver.py) and the native dqmc_main
(apps/dqmc_main.cpp) run one configuration against tests/fake_abi/fake_dqmc.c, a C-ABI
without a device whose answers depend on the walker, bin, tau and displacement, and
must write the same files and the same scalar results: the same bins per walker, the
same normalisation (MeasureHandler::normalize_stats, the dynamic sign), the same pooling
in walker order and the same analysis."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))

import dqmc_gb300 as dq  # noqa: E402
from dqmc_gb300 import io as dio  # noqa: E402
from dqmc_gb300 import run as drv  # noqa: E402

CONFIG = """
[Model]
    type = "RepulsiveHubbard"
[Lattice]
    %s
    momentum_list = "%s"
[MonteCarlo]
    beta = 1.0
    time_size = 6
    stabilization_pace = 3
[Measure]
    sweeps_warmup = 4
    bin_num = 5
    bin_size = 6
    sweeps_between_bins = 2
    observables = [ %s ]
"""


@pytest.fixture(scope="module")
def fake(tmp_path_factory):
    cc, cxx = shutil.which("gcc"), shutil.which("g++")
    if not cc or not cxx:
        pytest.skip("no C/C++ compiler")
    d = tmp_path_factory.mktemp("fake_abi")
    lib = d / "libdqmc_gb300.so"
    subprocess.run([cc, "-std=c99", "-shared", "-fPIC", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "fake_abi", "fake_dqmc.c"), "-o", str(lib), "-lm"], check=True)
    exe = d / "dqmc_main"
    subprocess.run([cxx, "-std=c++17", "-O2", os.path.join(ROOT, "dqmc-framework_gb300", "apps", "dqmc_main.cpp"),
                    "-L", str(d), "-ldqmc_gb300", "-Wl,-rpath," + str(d), "-o", str(exe)], check=True)
    return str(lib), str(exe)


def _numbers(path):
    return np.array([float(x) for x in open(path).read().split()])


SQUARE = 'cell = [ 4, 4 ]\n    momentum = "MPoint"'
CUBIC = 'type = "Cubic"\n    cell = [ 3, 3, 3 ]\n    momentum = "XPoint"'


@pytest.mark.parametrize("lattice,observables,klist,walkers", [
    (SQUARE, '"filling_number", "kinetic_energy", "s_wave_pairing_corr"', "KstarsAll", 2),  # device binning path
    (SQUARE, '"all"', "DeltaLine", 3),                                                       # dynamic path
    (SQUARE, '"density_of_states", "greens_functions"', "KstarsAll", 1),                   # dynamic only
    (CUBIC, '"all"', "LambdaLine", 2),  # cubic: 3-D momenta, no superfluid stiffness
])
def test_python_and_native_drivers_write_the_same_results(fake, tmp_path, monkeypatch, lattice, observables, klist,
                                                          walkers):
    lib, exe = fake
    cfg_text = CONFIG % (lattice, klist, observables)
    nsite = 27 if lattice == CUBIC else 16
    cfg_path = tmp_path / "config.toml"
    cfg_path.write_text(cfg_text)
    for who in ("py", "cpp"):  # each starts from the same fields file, which each writes back
        (tmp_path / f"fields_{who}.in").write_text(dio.format_fields([[(-1) ** (i + t) for i in range(nsite)]
                                                                       for t in range(6)]))
    # Python driver over the stand-in library
    monkeypatch.setattr(dq, "LIB_PATH", lib)
    monkeypatch.setattr(dq, "_lib", None)
    out_py = tmp_path / "py"
    import io as sio

    log = sio.StringIO()
    res = drv.run(dio.parse_config(cfg_text), str(out_py), walkers=walkers, seed=3,
                  fields_file=str(tmp_path / "fields_py.in"), log=log)
    # native driver over the same library
    out_cpp = tmp_path / "cpp"
    r = subprocess.run([exe, "-c", str(cfg_path), "-o", str(out_cpp), "-f", str(tmp_path / "fields_cpp.in"),
                        "--walkers", str(walkers), "--seed", "3"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    py_files = sorted(p.name for p in out_py.iterdir())
    assert py_files == sorted(p.name for p in out_cpp.iterdir())
    assert py_files, "no output"
    for name in py_files:
        a, b = _numbers(out_py / name), _numbers(out_cpp / name)
        assert a.shape == b.shape, name
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12, err_msg=name)
    assert (tmp_path / "fields_py.in").read_text() == (tmp_path / "fields_cpp.in").read_text()
    # the scalar summary: the same names, means and errors
    def summary(text):
        out = {}
        for line in text.splitlines():
            if " pm " in line and "->" in line:
                desc, rest = line.split("->")
                m, e = rest.split("pm")
                out[desc.strip()] = (float(m), float(e))
        return out

    s_py, s_cpp = summary(log.getvalue()), summary(r.stdout)
    assert s_py.keys() == s_cpp.keys() and len(s_py) == len(res)
    for k in s_py:
        np.testing.assert_allclose(s_py[k], s_cpp[k], rtol=1e-11, atol=1e-12, err_msg=k)
    assert ">> Maximum of the wrapping error: %.5e" % (1e-9 * walkers) in r.stdout
