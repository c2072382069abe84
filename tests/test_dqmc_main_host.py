"""The native dqmc_main (apps/dqmc_main.cpp) without a GPU: its --dry-run does all the host
work of the reference's main program (src/dqmc_main.cpp): the TOML configuration by the
reference's rules, the start-up lines and the parameter block, kstars.out and
tgrids.out, and the fields file read and written back.  Pinned against the reference's
example output (tests/golden/io_formats.json) and cross-checked with the Python reader
and writers (dqmc_gb300.io) on the same configurations."""
import hashlib
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
from dqmc_gb300 import io as dio  # noqa: E402

FIX = json.load(open(os.path.join(HERE, "golden", "io_formats.json")))

EXAMPLE_CONFIG = """
## a configuration in the reference's layout: comments, a sub-table, a multi-line array
[Model]
    type = "AttractiveHubbard"   # the example's model
    [Model.Params]
    hopping_t = 1.0
    onsite_u = 4.0
    chemical_potential = 0.0
[Lattice]
    type = "Square"
    cell = [ 8, 8 ]
    momentum = "MPoint"
    momentum_list = "KstarsAll"
[CheckerBoard]
    whether_or_not = false
[MonteCarlo]
    beta = 8.0
    time_size = 160
    stabilization_pace = 10
[Measure]
    sweeps_warmup = 512
    bin_num = 20
    bin_size = 100
    sweeps_between_bins = 20
    observables = [
        "all",   # every observable
    ]
"""


@pytest.fixture(scope="module")
def exe():
    import __graft_entry__ as g

    g.build_library()
    path = os.path.join(ROOT, "dqmc-framework_gb300", "lib", "dqmc_main")
    assert os.path.exists(path)
    return path


def _run(exe, args, cwd=None):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    return subprocess.run([exe] + args, capture_output=True, text=True, env=env, timeout=120, cwd=cwd)


def _sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def _init_block(stdout):
    start = stdout.index("   Model:")
    return stdout[start:]


def test_example_dry_run_is_byte_identical(exe, tmp_path, example_fixture):
    cfg = tmp_path / "config.toml"
    cfg.write_text(EXAMPLE_CONFIG)
    fields = tmp_path / "fields.in"
    fields.write_text(dio.format_fields(example_fixture["fields"].tolist()))
    out = tmp_path / "out" / "nested"  # created as dqmc_main creates its output folder
    r = _run(exe, ["--dry-run", "-c", str(cfg), "-o", str(out), "-f", str(fields), "--walkers", "10"])
    assert r.returncode == 0, r.stderr
    assert _sha(out / "kstars.out") == FIX["files"]["kstars.out"]["sha256"]
    assert _sha(out / "tgrids.out") == FIX["files"]["tgrids.out"]["sha256"]
    assert _sha(fields) == FIX["files"]["fields.out"]["sha256"]  # read and written back unchanged
    assert ">> Configurations of the bosonic fields read from the input config file.\n" in r.stdout
    assert _init_block(r.stdout) == FIX["log"]["init_info"] + "\n"


CONFIGS = [
    ('[Lattice]\ncell = [4, 4]\n[Measure]\nobservables = ["none"]\n', 1),
    ('[Model]\ntype = "RepulsiveHubbard"\n[Model.Params]\nonsite_u = 6\nchemical_potential = -0.25\n'
     '[Lattice]\ncell = [6, 6]\nmomentum = "XPoint"\nmomentum_list = "Gamma2X2M2GammaLoop"\n'
     '[CheckerBoard]\nwhether_or_not = true\n[MonteCarlo]\nbeta = 3\ntime_size = 60.0\nstabilization_pace = 6\n'
     '[Measure]\nsweeps_warmup = 0\nbin_num = 7\nbin_size = 10\nsweeps_between_bins = 2\n'
     'observables = ["double_occupancy", "greens_functions"]\n', 3),
    ('[Lattice]\ntype = "Cubic"\ncell = [4, 4, 4]\nmomentum = "RPoint"\nmomentum_list = "LambdaLine"\n'
     '[Measure]\nobservables = ["all"]\n', 2),
]


@pytest.mark.parametrize("text,walkers", CONFIGS)
def test_native_and_python_readers_agree(exe, tmp_path, text, walkers):
    """The same configuration through toml_config.hpp and dqmc_gb300.io.parse_config gives the
    same parameter block and the same k-star file."""
    cfg_path = tmp_path / "c.toml"
    cfg_path.write_text(text)
    r = _run(exe, ["--dry-run", "--config", str(cfg_path), "--output", str(tmp_path), "--walkers", str(walkers)])
    assert r.returncode == 0, r.stderr
    cfg = dio.parse_config(text)
    assert _init_block(r.stdout) == dio.format_init_info(cfg, walkers)
    assert (tmp_path / "kstars.out").read_text() == dio.format_kstars(cfg.L, cfg.dim)
    assert (tmp_path / "tgrids.out").read_text() == dio.format_tgrids(cfg.beta, cfg.time_size)


BAD = [
    '[Model]\ntype = "Kondo"\n[Lattice]\ncell = [4, 4]\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ncell = [4, 0]\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ncell = [4, 4]\n',
    '[Lattice]\ncell = [4, 4]\n[Measure]\nobservables = ["magic"]\n',
    '[Lattice]\ntype = "Honeycomb"\ncell = [4, 4]\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ntype = "Cubic"\ncell = [4, 4, 4]\n[CheckerBoard]\nwhether_or_not = true\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ncell = [4, 4]\nmomentum = "RPoint"\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ncell = [4, 4\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ncell = [4, 4]\ncell = [6, 6]\n[Measure]\nobservables = ["all"]\n',
]


@pytest.mark.parametrize("text", BAD)
def test_native_reader_rejects_what_the_reference_rejects(exe, tmp_path, text):
    cfg_path = tmp_path / "bad.toml"
    cfg_path.write_text(text)
    r = _run(exe, ["--dry-run", "-c", str(cfg_path), "-o", str(tmp_path)])
    assert r.returncode == 1 and r.stderr.startswith("dqmc_main: "), (r.stdout, r.stderr)


def test_options_fields_and_device(exe, tmp_path):
    cfg_path = tmp_path / "c.toml"
    cfg_path.write_text('[Lattice]\ncell = [4, 4]\n[MonteCarlo]\ntime_size = 6\n[Measure]\nobservables = ["all"]\n')
    assert _run(exe, ["--bogus"]).returncode == 1
    assert "undefined options" in _run(exe, ["-c"]).stderr
    bad_fields = tmp_path / "f.in"
    bad_fields.write_text(f"{6:20d}{16:20d}\n{9:20d}{0:20d}{1.0:20.1f}\n")
    r = _run(exe, ["--dry-run", "-c", str(cfg_path), "-o", str(tmp_path), "-f", str(bad_fields)])
    assert r.returncode == 1 and "outside" in r.stderr
    # without --dry-run the run needs the device: without one it fails loudly, no CPU fallback
    r = _run(exe, ["-c", str(cfg_path), "-o", str(tmp_path / "o")])
    assert r.returncode == 1 and "no CUDA device" in r.stderr
    cubic = tmp_path / "cubic.toml"
    cubic.write_text('[Lattice]\ntype = "Cubic"\ncell = [4, 4, 4]\n[Measure]\nobservables = ["all"]\n')
    r = _run(exe, ["-c", str(cubic), "-o", str(tmp_path / "o")])
    assert r.returncode == 1 and "no CUDA device" in r.stderr  # the cubic lattice runs on the device too
