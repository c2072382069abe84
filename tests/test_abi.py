"""C-ABI checks that need no GPU: the library loads, exports every symbol the
public header declares, and rejects bad arguments before touching a device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dq():
    import __graft_entry__ as g

    g.build_library()
    import dqmc_gb300

    dqmc_gb300.load()
    return dqmc_gb300


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dqmc_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(dq):
    lib = ctypes.CDLL(dq.LIB_PATH)
    declared = _declared("dqmc_gb300.h")
    assert declared, "no declarations parsed"
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(dq.EXPORTS) == sorted(declared)


def test_abi_version(dq):
    assert dq.load().dqmc_abi_version() == 3


def test_walker_desc_layout_matches_header(dq):
    """dqmc_walker_desc as the header lays it out: the lattice field last, after the seed."""
    d = dq._Desc
    assert d.lattice.offset == d.seed.offset + 8 and ctypes.sizeof(d) == d.lattice.offset + 8
    assert dq.WalkerDesc(L=5, lattice=dq.CUBIC).N == 125 and dq.WalkerDesc(L=5).N == 25


@pytest.mark.parametrize(
    "kw, msg",
    [
        (dict(L=1), "side"),
        (dict(L=33), "exceeds"),
        (dict(L=3, checkerboard=True), "even"),
        (dict(Lt=0), "Lt"),
        (dict(pace=0), "pace"),
        (dict(beta=-1.0), "beta"),
        (dict(model=7), "model"),
        (dict(L=4, momentum_index=99), "momentum"),
        (dict(L=4, lattice=2), "lattice"),
        (dict(L=11, lattice=1), "exceeds"),  # 1331 sites
        (dict(L=4, lattice=1, checkerboard=True), "square lattice only"),
        (dict(L=4, lattice=1, momentum_index=10), "momentum"),  # 10 k stars of the 4^3 lattice
    ],
)
def test_bad_arguments_rejected_before_device(dq, kw, msg):
    with pytest.raises(dq.DqmcError) as e:
        dq.Batch([dq.WalkerDesc(**kw)])
    assert "status 1" in str(e.value) and msg in str(e.value)


def test_null_batch_calls_fail_cleanly(dq):
    L = dq.load()
    assert L.dqmc_init_greens(None) == 1
    assert L.dqmc_sweep_0_to_beta(None, 0) == 1
    assert L.dqmc_batch_destroy(None) == 0


def test_no_cpu_fallback_without_gpu(dq):
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(dq.DqmcError) as e:
        dq.Batch([dq.WalkerDesc()])
    assert "status 2" in str(e.value)


def test_python_setters_check_sizes_before_the_library_reads(dq):
    """set_fields / set_green hand a raw pointer to the library, which reads Lt * N bytes or
    N * N doubles: the binding refuses arrays of another size and walkers outside the batch."""
    import numpy as np

    b = dq.Batch.__new__(dq.Batch)  # no device: only the host-side checks run
    b.h = None
    b.walkers = [dq.WalkerDesc(L=4, Lt=8)]
    with pytest.raises(ValueError):
        b.set_fields(0, np.ones((8, 15), dtype=np.int8))
    with pytest.raises(ValueError):
        b.set_green(0, 0, np.eye(15))
    with pytest.raises(IndexError):
        b.set_fields(1, np.ones((8, 16), dtype=np.int8))
    with pytest.raises(IndexError):
        b.green(-1, 0)


def test_header_is_plain_c_and_links(dq, tmp_path):
    """include/dqmc_gb300.h is what an FFI binding (cgo, ctypes, JNI) includes: it must compile as
    strict C99 and a C program must link against the library with it."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    src.write_text('#include "dqmc_gb300.h"\n'
                   "int main(void) { dqmc_batch_options o = {0}; (void)o;\n"
                   "  return dqmc_abi_version() == DQMC_ABI_VERSION ? 0 : 1; }\n")
    inc = os.path.join(ROOT, "include")
    libdir = os.path.dirname(dq.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-I", inc, str(src)],
                   check=True)
    exe = tmp_path / "abi"
    subprocess.run([cc, "-std=c99", "-I", inc, str(src), "-L", libdir, "-ldqmc_gb300", "-Wl,-rpath," + libdir,
                    "-o", str(exe)], check=True)
    assert subprocess.run([str(exe)]).returncode == 0  # dqmc_abi_version needs no device


def test_cpp_driver_fails_loudly_without_a_device(dq):
    """The C++ driver built over include/dqmc_gb300.hpp exits non-zero with the library's
    message when no GPU is visible (no CPU fallback), and rejects unknown arguments."""
    import subprocess

    exe = os.path.join(os.path.dirname(dq.LIB_PATH), "dqmc_run")
    if not os.path.exists(exe):
        pytest.skip("driver not built")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([exe, "L=4", "walkers=2"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "no CUDA device" in (r.stdout + r.stderr)
    r = subprocess.run([exe, "bogus=1"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "unknown argument" in (r.stdout + r.stderr)
    # the cubic lattice reaches the library (which then needs the device); bad lattices stop earlier
    r = subprocess.run([exe, "lattice=cubic", "L=4"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "no CUDA device" in (r.stdout + r.stderr)
    r = subprocess.run([exe, "lattice=honeycomb"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "square or cubic" in (r.stdout + r.stderr)
    r = subprocess.run([exe, "lattice=cubic", "L=1"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "Cubic" in (r.stdout + r.stderr)


def test_cpp_mirror_analysis_matches_python(tmp_path):
    """MeasureHandler::analyse_stats of include/dqmc_gb300.hpp and dqmc_gb300.io.analyse_bins
    (both Observable::analyse, include/measure/observable.h:169-211) agree on the same bins."""
    import shutil
    import subprocess

    import numpy as np

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    rng = np.random.default_rng(11)
    bins = rng.normal(0.5, 0.2, (7, 9))
    src = tmp_path / "analyse.cpp"
    rows = ",\n".join("{" + ", ".join(repr(float(v)) for v in b) + "}" for b in bins)
    src.write_text('#include <cstdio>\n#include "dqmc_gb300.hpp"\n'
                   "int main() {\n  dqmc_gb300::MeasureHandler m;\n"
                   f"  m.bins = {{{rows}}};\n  m.analyse_stats();\n"
                   '  for (int k = 0; k < DQMC_NUM_OBS; ++k) std::printf("%.17g %.17g\\n", m.mean[k], m.error[k]);\n}\n')
    exe = tmp_path / "analyse"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, timeout=120)
    out = np.array([[float(x) for x in l.split()] for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                                           check=True).stdout.splitlines()])
    import sys

    sys.path.insert(0, os.path.join(ROOT, "dqmc-framework_gb300"))
    from dqmc_gb300 import io as dio

    mean, err = dio.analyse_bins(bins)
    np.testing.assert_allclose(out[:, 0], mean, rtol=1e-14)
    np.testing.assert_allclose(out[:, 1], err, rtol=1e-12)
