"""Reference-compatible configuration parsing and text output (dqmc_gb300.io).

The writers are pinned to the reference's own example output (fixture
tests/golden/io_formats.json, made by make_io_fixture.py from
example/output/*.out): kstars.out, tgrids.out and fields.out are rebuilt from the
example's parameters and field configuration and must be byte-identical; the
rows of the observable files are re-formatted field by field.
"""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "dqmc-framework_gb300"))

from dqmc_gb300 import io as dio  # noqa: E402  (host code only; no device library needed)

FIX = json.load(open(os.path.join(HERE, "golden", "io_formats.json")))["files"]
EX = json.load(open(os.path.join(HERE, "golden", "example_8x8.json")))


def _sha(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()


def test_kstars_and_tgrids_are_byte_identical():
    assert _sha(dio.format_kstars(EX["L"])) == FIX["kstars.out"]["sha256"]
    assert _sha(dio.format_tgrids(EX["beta"], EX["Lt"])) == FIX["tgrids.out"]["sha256"]


def test_fields_file_round_trip_is_byte_identical():
    bits = np.unpackbits(np.frombuffer(bytes.fromhex(EX["fields_packed_hex"]), dtype=np.uint8))
    fields = np.where(bits[: EX["Lt"] * EX["N"]].reshape(EX["Lt"], EX["N"]) > 0, 1, -1)
    text = dio.format_fields(fields.tolist())
    assert _sha(text) == FIX["fields.out"]["sha256"]
    lt, n, back = dio.parse_fields(text)
    assert (lt, n) == (EX["Lt"], EX["N"]) and (np.array(back) == fields).all()


@pytest.mark.parametrize("name", ["dos.out", "dss.out", "greens.out", "swave.out", "dos.bins.out",
                                  "greens.bins.out", "swave.bins.out"])
def test_observable_rows_reformat_identically(name):
    for line in FIX[name]["head"]:
        if not line:
            continue
        assert len(line) % 20 == 0
        fields = [line[k:k + 20] for k in range(0, len(line), 20)]
        for f in fields:
            tok = f.strip()
            if "." in tok:
                assert dio._f(float(tok)) == f
            else:
                assert dio._d(int(tok)) == f


def test_writers_layout():
    mean, err = np.array([0.5, 0.25]), np.array([0.01, 0.02])
    v = dio.format_vector(mean, err).splitlines()
    assert v[0] == dio._d(2) and v[2] == dio._d(1) + dio._f(0.25) + dio._f(0.02) + dio._f(0.08)
    m = dio.format_matrix([[1.0, 2.0]], [[0.1, 0.2]]).splitlines()
    assert m[0] == dio._d(1) + dio._d(2) and m[2].startswith(dio._d(0) + dio._d(1) + dio._f(2.0))
    bins = np.arange(6.0).reshape(3, 2)
    bv = dio.format_bins_vector(bins).splitlines()
    assert bv[0] == dio._d(3) + dio._d(2) and bv[-1] == dio._d(2) + dio._d(1) + dio._f(5.0)
    bm = dio.format_bins_matrix(bins[:, None, :]).splitlines()
    assert bm[0] == dio._d(3) + dio._d(1) + dio._d(2) and len(bm) == 7
    assert dio.format_summary_line("Filling number", 0.5, 0.01) == \
        f"{'Filling number':>30s}{'->':>7s}{0.5:20.12f}  pm  {0.01:.12f}\n"


def test_analyse_bins_matches_the_reference_formula():
    rng = np.random.default_rng(1)
    b = rng.standard_normal((20, 3))
    mean, err = dio.analyse_bins(b)
    np.testing.assert_allclose(mean, b.mean(axis=0), rtol=1e-14)
    ref = np.sqrt((b ** 2).mean(axis=0) - b.mean(axis=0) ** 2) / np.sqrt(19)
    np.testing.assert_allclose(err, ref, rtol=1e-12)


CONFIG = """
[Model]
    type = "AttractiveHubbard"
    [Model.Params]
    hopping_t = 1.0
    onsite_u = 4.0
    chemical_potential = -0.5
[Lattice]
    type = "Square"
    cell = [ 6, 6 ]
    momentum = "XPoint"
    momentum_list = "KstarsAll"
[CheckerBoard]
    whether_or_not = false
[MonteCarlo]
    beta = 4.0
    time_size = 80
    stabilization_pace = 8
[Measure]
    sweeps_warmup = 100
    bin_num = 10
    bin_size = 20
    sweeps_between_bins = 4
    observables = [ "all" ]
"""


def test_parse_config_keys_defaults_and_keywords():
    c = dio.parse_config(CONFIG)
    assert (c.model, c.hopping_t, c.onsite_u, c.chemical_potential) == ("AttractiveHubbard", 1.0, 4.0, -0.5)
    assert (c.L, c.momentum, c.checkerboard) == (6, "XPoint", False)
    assert (c.beta, c.time_size, c.stabilization_pace) == (4.0, 80, 8)
    assert (c.sweeps_warmup, c.bin_num, c.bin_size, c.sweeps_between_bins) == (100, 10, 20, 4)
    assert c.observables == dio.ALL_OBSERVABLES
    assert c.equaltime == dio.EQUALTIME_OBSERVABLES and c.dynamic == dio.DYNAMIC_OBSERVABLES
    # defaults of DqmcInitializer::parse_toml_config where a key is absent
    d = dio.parse_config('[Lattice]\ncell = [4, 4]\n[Measure]\nobservables = ["none"]\n')
    assert (d.model, d.onsite_u, d.beta, d.time_size, d.stabilization_pace) == ("RepulsiveHubbard", 4.0, 4.0, 80, 10)
    assert (d.sweeps_warmup, d.bin_num, d.bin_size, d.sweeps_between_bins) == (512, 20, 100, 20)
    assert d.observables == []
    # k stars and high-symmetry points of the 6x6 lattice (Square::initial_symmetry_points)
    ks = dio.kstars(6)
    assert len(ks) == 10 and ks[0] == (0.0, 0.0)
    assert dio.momentum_index(6, "MPoint") == 9 and dio.momentum_index(6, "XPoint") == 6
    assert ks[6] == pytest.approx((np.pi, 0.0)) and ks[9] == pytest.approx((np.pi, np.pi))


@pytest.mark.parametrize("bad", [
    '[Model]\ntype = "Kondo"\n[Lattice]\ncell = [4, 4]\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ncell = [4, 0]\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ncell = [4, 4]\n',
    '[Lattice]\ncell = [4, 4]\n[Measure]\nobservables = ["magic"]\n',
    '[Lattice]\ntype = "Honeycomb"\ncell = [4, 4]\n[Measure]\nobservables = ["all"]\n',
])
def test_parse_config_rejects_what_the_reference_rejects(bad):
    with pytest.raises(ValueError):
        dio.parse_config(bad)


CUBIC = """
[Model]
    type = "RepulsiveHubbard"
[Lattice]
    type = "Cubic"
    cell = [4, 4, 4]
    momentum = "RPoint"
    momentum_list = "LambdaLine"
[Measure]
    observables = [ "all" ]
"""


def test_parse_cubic_config():
    """Cubic tables of DqmcInitializer::parse_toml_config (dqmc_initializer.cpp:118-150,
    233-237, 293-327): three equal sides, R point, cubic lines, no superfluid stiffness."""
    c = dio.parse_config(CUBIC)
    assert (c.lattice, c.cell, c.L, c.dim) == ("Cubic", (4, 4, 4), 4, 3)
    assert "superfluid_stiffness" not in c.observables
    assert c.observables == [o for o in dio.ALL_OBSERVABLES if o != "superfluid_stiffness"]
    assert dio.momentum_index(4, c.momentum, 3) == len(dio.kstars(4, 3)) - 1
    with pytest.raises(ValueError):
        dio.momentum_index(4, "RPoint")  # not a square-lattice point
    with pytest.raises(ValueError):
        dio.momentum_list_indices(4, "Gamma2X2M2GammaLoop", 3)  # not a cubic-lattice list


@pytest.mark.parametrize("bad", [
    '[Lattice]\ntype = "Cubic"\ncell = [4, 4]\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ntype = "Cubic"\ncell = [4, 4, 3]\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ntype = "Cubic"\ncell = [4, 4, 4]\n[CheckerBoard]\nwhether_or_not = true\n[Measure]\nobservables = ["all"]\n',
    '[Lattice]\ntype = "Square"\ncell = [4, 4, 4]\n[Measure]\nobservables = ["all"]\n',
])
def test_parse_cubic_rejects_what_the_reference_rejects(bad):
    with pytest.raises(ValueError):
        dio.parse_config(bad)


@pytest.mark.parametrize("L", [2, 3, 4, 5, 6, 7, 8])
def test_cubic_kstars_points_and_lines(L):
    """Cubic::initial_index2momentum_table and initial_symmetry_points (cubic.cpp:47-183):
    the count's closed form, the points X, M, R and the six lines lying where they should."""
    ks = np.array(dio.kstars(L, 3))
    h = L // 2 + 1
    assert len(ks) == round(h * (h + 1) * (2 * h + 1) / 12 + h * (h + 1) / 4)
    pi = np.pi
    first = ks[0, 0]  # 0 for even L; the reference's grid is offset by pi for odd L
    pts = {n: ks[dio.momentum_index(L, n, 3)] for n in ("GammaPoint", "XPoint", "MPoint", "RPoint")}
    np.testing.assert_allclose(pts["GammaPoint"], [first] * 3, atol=1e-12)
    np.testing.assert_allclose(pts["XPoint"], [pi, first, first], atol=1e-12)
    np.testing.assert_allclose(pts["MPoint"], [pi, pi, first], atol=1e-12)
    np.testing.assert_allclose(pts["RPoint"], [pi, pi, pi], atol=1e-12)
    line = lambda n: ks[dio.momentum_list_indices(L, n, 3)]
    d, z, s = line("DeltaLine"), line("ZLine"), line("SigmaLine")
    lam, sl, tl = line("LambdaLine"), line("SLine"), line("TLine")
    for pts_, fixed in ((d, [1, 2]), (z, [2]), (s, [2]), (sl, []), (tl, [])):
        for a in fixed:
            np.testing.assert_allclose(pts_[:, a], first, atol=1e-12)
    np.testing.assert_allclose(d[:, 0], np.sort(d[:, 0]))                       # Gamma -> X
    np.testing.assert_allclose(z[:, 0], pi, atol=1e-12)                         # X -> M
    np.testing.assert_allclose(s[:, 0], s[:, 1])                                # Gamma -> M
    np.testing.assert_allclose(lam[:, 0], lam[:, 1]); np.testing.assert_allclose(lam[:, 1], lam[:, 2])  # Gamma -> R
    np.testing.assert_allclose(sl[:, 0], pi, atol=1e-12); np.testing.assert_allclose(sl[:, 1], sl[:, 2])  # X -> R
    np.testing.assert_allclose(tl[:, :2], pi, atol=1e-12)                       # M -> R
    for seq in (d[:, 0], z[:, 1], s[:, 0], lam[:, 0], sl[:, 1], tl[:, 2]):
        assert len(seq) == L // 2 + 1 and (np.diff(seq) > 0).all()


def test_cubic_kstars_file_layout():
    """DqmcIO::output_k_stars writes SpaceDim components per k star."""
    text = dio.format_kstars(4, 3)
    lines = text.splitlines()
    assert int(lines[0]) == len(dio.kstars(4, 3)) == 10
    assert all(len(l) == 80 for l in lines[1:])  # index + kx + ky + kz, 20 columns each
    assert dio.format_kstars(4) == dio.format_kstars(4, 2)


def test_cubic_kstars_agree_with_the_oracle(oracle_mod):
    w = oracle_mod.Walker(L=5, Lt=4, pace=2, lattice=oracle_mod.CUBIC)
    ks = dio.kstars(5, 3)
    assert len(ks) == w.num_k_stars()
    for k, v in enumerate(ks):
        np.testing.assert_array_equal(w.k_star(k), v)


LOG = json.load(open(os.path.join(HERE, "golden", "io_formats.json")))["log"]
EXAMPLE_CONFIG = """
[Model]
    type = "AttractiveHubbard"
    [Model.Params]
    hopping_t = 1.0
    onsite_u = 4.0
    chemical_potential = 0.0
[Lattice]
    type = "Square"
    cell = [8, 8]
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
    observables = ["all"]
"""


def test_terminal_blocks_are_byte_identical_to_the_reference_log():
    """DqmcIO::output_init_info, output_ending_info and dqmc_main's scalar summary rebuilt from
    the example's parameters (10 MPI ranks) and logged numbers equal example/log.out."""
    cfg = dio.parse_config(EXAMPLE_CONFIG)
    assert dio.format_init_info(cfg, 10) == LOG["init_info"] + "\n"
    assert dio.format_ending_info(102.03, 1.08516e-08) == LOG["ending_info"] + "\n"
    names = {v: k for k, v in dio.DESCRIPTIONS.items()}
    results = {}
    for line in LOG["summary"].splitlines():
        if "->" in line:
            desc, rest = line.split("->")
            mean, err = rest.split("pm")
            results[names[desc.strip()]] = (float(mean), float(err))
    assert len(results) == 11
    assert dio.format_summary(results) == LOG["summary"]


def test_ending_info_time_formats():
    """d/h/m/s forms of DqmcIO::output_ending_info."""
    assert ">> The simulation finished in 5.25 s." in dio.format_ending_info(5.25, 0.0)
    assert ">> The simulation finished in 2 h 0 m 1.50 s." in dio.format_ending_info(7201.5, 0.0)
    assert ">> The simulation finished in 1 d 1 h 1 m 1.00 s." in dio.format_ending_info(90061.0, 0.0)
    cubic = dio.parse_config('[Lattice]\ntype = "Cubic"\ncell = [4, 4, 4]\nmomentum = "RPoint"\n'
                             '[Measure]\nobservables = ["filling_number"]\n')
    info = dio.format_init_info(cubic, 3)
    assert "   Lattice: Cubic lattice\n" in info and "(1.00, 1.00, 1.00) pi" in info and "4 * 4 * 4" in info
    assert dio._param("Number of bins", "21") in info and dio._param("Dynamical measure", "False") in info
