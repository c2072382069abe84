"""Reference-compatible configuration and text output.

Reads the reference's TOML configuration (DqmcInitializer::parse_toml_config,
src/dqmc_initializer.cpp:27-338: the same tables, keys and defaults) and writes
its text files (DqmcIO, include/dqmc_io.h:267-629: observables as means and
errors or raw bins, k stars, imaginary-time grids, bosonic fields) in the same
formats, so that existing configurations and analysis scripts work unchanged.
Host code only: nothing here touches the device.
"""
from __future__ import annotations

import math
import tomllib
from dataclasses import dataclass, field

# MeasureHandler::ObservableAll (src/measure/measure_handler.cpp), equal-time then dynamic
EQUALTIME_OBSERVABLES = [
    "filling_number", "double_occupancy", "kinetic_energy", "momentum_distribution", "local_spin_corr",
    "spin_density_structure_factor", "charge_density_structure_factor", "s_wave_pairing_corr",
]
DYNAMIC_OBSERVABLES = ["greens_functions", "density_of_states", "superfluid_stiffness",
                       "dynamic_spin_susceptibility"]
ALL_OBSERVABLES = EQUALTIME_OBSERVABLES + DYNAMIC_OBSERVABLES


@dataclass
class RunConfig:
    """The parsed configuration (reference defaults where a key is absent)."""
    model: str = "RepulsiveHubbard"
    hopping_t: float = 1.0
    onsite_u: float = 4.0
    chemical_potential: float = 0.0
    lattice: str = "Square"   # "Square" or "Cubic"
    cell: tuple = (4, 4)
    momentum: str = ""
    momentum_list: str = ""
    checkerboard: bool = False
    beta: float = 4.0
    time_size: int = 80
    stabilization_pace: int = 10
    sweeps_warmup: int = 512
    bin_num: int = 20
    bin_size: int = 100
    sweeps_between_bins: int = 20
    observables: list = field(default_factory=list)

    @property
    def L(self) -> int:
        return self.cell[0]

    @property
    def dim(self) -> int:
        return len(self.cell)

    @property
    def equaltime(self) -> list:
        return [o for o in self.observables if o in EQUALTIME_OBSERVABLES]

    @property
    def dynamic(self) -> list:
        return [o for o in self.observables if o in DYNAMIC_OBSERVABLES]


def parse_config(text: str) -> RunConfig:
    """DqmcInitializer::parse_toml_config on a TOML string.  Raises ValueError where the
    reference exits (unknown model or lattice, bad cell, checkerboard off the square lattice,
    missing observable list, unknown momentum names when they are used).  The reference also
    exits when `momentum` or `momentum_list` is absent; here they default to the last k star,
    (pi, ..., pi), and to every k star."""
    c = tomllib.loads(text)
    m, lat = c.get("Model", {}), c.get("Lattice", {})
    p, mc, me = m.get("Params", {}), c.get("MonteCarlo", {}), c.get("Measure", {})
    cfg = RunConfig()
    cfg.model = m.get("type", "RepulsiveHubbard")
    if cfg.model not in ("RepulsiveHubbard", "AttractiveHubbard"):
        raise ValueError(f"undefined model type '{cfg.model}'")
    cfg.hopping_t = float(p.get("hopping_t", 1.0))
    cfg.onsite_u = float(p.get("onsite_u", 4.0))
    cfg.chemical_potential = float(p.get("chemical_potential", 0.0))
    cfg.lattice = lat.get("type", "Square")
    dims = {"Square": (2, "2d square", "two"), "Cubic": (3, "3d cubic", "three")}
    if cfg.lattice not in dims:  # Honeycomb: left unimplemented by the reference
        raise ValueError(f"undefined lattice type '{cfg.lattice}'")
    dim, what, count = dims[cfg.lattice]
    cell = lat.get("cell")
    if not isinstance(cell, list) or len(cell) != dim or any((not isinstance(v, int)) or v < 1 for v in cell):
        raise ValueError(f"the input cell of {what} lattice should be a vector containing {count} positive integers")
    if len(set(cell)) != 1:  # Square/Cubic::set_lattice_params assert equal sides
        raise ValueError(f"the {what} lattice must have equal sides")
    cfg.cell = tuple(cell)
    cfg.momentum = lat.get("momentum", "")
    cfg.momentum_list = lat.get("momentum_list", "")
    cfg.checkerboard = bool(c.get("CheckerBoard", {}).get("whether_or_not", False))
    if cfg.checkerboard and cfg.lattice != "Square":
        raise ValueError("the checkerboard method is currently only implemented for 2d square lattice")
    cfg.beta = float(mc.get("beta", 4.0))
    cfg.time_size = int(mc.get("time_size", 80))
    cfg.stabilization_pace = int(mc.get("stabilization_pace", 10))
    cfg.sweeps_warmup = int(me.get("sweeps_warmup", 512))
    cfg.bin_num = int(me.get("bin_num", 20))
    cfg.bin_size = int(me.get("bin_size", 100))
    cfg.sweeps_between_bins = int(me.get("sweeps_between_bins", 20))
    obs = me.get("observables")
    if not isinstance(obs, list) or not all(isinstance(o, str) for o in obs):
        raise ValueError("undefined observables, please check the config")
    if len(obs) == 1 and obs[0] in ("all", "All"):
        obs = list(ALL_OBSERVABLES)
    elif len(obs) == 1 and obs[0] in ("none", "None"):
        obs = []
    for o in obs:
        if o not in ALL_OBSERVABLES:
            raise ValueError(f"unsupported observable '{o}'")
    if cfg.lattice != "Square":  # a square-lattice observable (dqmc_initializer.cpp:233-237)
        obs = [o for o in obs if o != "superfluid_stiffness"]
    cfg.observables = obs
    return cfg


def load_config(path: str) -> RunConfig:
    with open(path, encoding="utf-8") as f:
        return parse_config(f.read())


# ---- lattice tables (src/lattice/square.cpp:42-145, src/lattice/cubic.cpp:47-183) ----
def kstars(L: int, dim: int = 2) -> list:
    """The inequivalent momenta (k stars) of the L x L square or L x L x L cubic lattice, in
    the reference's order (the cubic ones fill the tetrahedron (0,0,0), (pi,0,0), (pi,pi,0),
    (pi,pi,pi) with kz outermost)."""
    m = lambda i: i / L * 2 * math.pi - math.pi
    lo = math.ceil(L / 2)
    if dim == 2:
        return [(m(i), m(j)) for i in range(lo, L + 1) for j in range(lo, i + 1)]
    return [(m(i), m(j), m(k)) for k in range(lo, L + 1) for i in range(k, L + 1) for j in range(k, i + 1)]


def _points(L: int, dim: int) -> dict:
    """Square/Cubic::initial_symmetry_points: indices of the high-symmetry points."""
    h = L // 2
    m_point = (h + 1) * (h + 2) // 2 - 1  # the last k star of the kz = 0 plane
    pts = {"GammaPoint": 0, "XPoint": m_point - h, "MPoint": m_point}
    if dim == 3:
        pts["RPoint"] = len(kstars(L, 3)) - 1
    return pts


def momentum_index(L: int, name: str, dim: int = 2) -> int:
    """Index of a high-symmetry point among the k stars: GammaPoint, XPoint, MPoint, and on
    the cubic lattice RPoint."""
    pts = _points(L, dim)
    if name not in pts:
        raise ValueError(f"undefined momentum '{name}' for the {'2d square' if dim == 2 else '3d cubic'} lattice "
                         f"({', '.join(pts)})")
    return pts[name]


def momentum_list_indices(L: int, name: str, dim: int = 2) -> list:
    """k-star indices of a momentum list (Square/Cubic::initial_symmetry_points and the
    initializer's momentum_list options): KstarsAll, DeltaLine, ZLine, SigmaLine, and
    Gamma2X2M2GammaLoop (square) or LambdaLine, SLine, TLine (cubic); a single point name
    gives that point."""
    nk = len(kstars(L, dim))
    h = L // 2
    pts = _points(L, dim)
    xp, mp = pts["XPoint"], pts["MPoint"]
    lines = {"KstarsAll": list(range(nk)), "DeltaLine": [i * (i + 1) // 2 for i in range(h + 1)],
             "ZLine": [xp + i for i in range(h + 1)], "SigmaLine": [i * (i + 3) // 2 for i in range(h + 1)]}
    if dim == 2:
        lines["Gamma2X2M2GammaLoop"] = ([i * (i + 1) // 2 for i in range(h)] + [xp + i for i in range(h)] +
                                        [i * (i + 3) // 2 for i in range(h, 0, -1)])
    else:  # cubic.cpp:160-182: each step skips one kz plane of the tetrahedron
        lam, sl, tl = [0], [xp], [mp]
        for i in range(1, h + 1):
            lam.append(lam[-1] + (h + 2 - i) * (h + 3 - i) // 2)
            sl.append(sl[-1] + (h + 1 - i) * (h + 2 - i) // 2 + 1)
            tl.append(tl[-1] + (h + 1 - i) * (h + 2 - i) // 2)
        lines.update(LambdaLine=lam, SLine=sl, TLine=tl)
    if name in lines:
        return lines[name]
    if name in pts:
        return [pts[name]]
    raise ValueError(f"undefined momentum list '{name}' ({', '.join(list(lines) + list(pts))})")


# ---- text formats (boost::format "%| 20.10f|" etc. of include/dqmc_io.h) ------------
def _f(v: float, prec: int = 10) -> str:
    return f"{v:20.{prec}f}"


def _d(v: int) -> str:
    return f"{v:20d}"


def format_scalar(mean: float, err: float) -> str:
    rel = err / mean if mean != 0 else math.inf
    return _f(mean) + _f(err) + _f(rel) + "\n"


def format_vector(mean, err) -> str:
    lines = [_d(len(mean)) + "\n"]
    for i, (m, e) in enumerate(zip(mean, err)):
        rel = e / m if m != 0 else math.inf
        lines.append(_d(i) + _f(m) + _f(e) + _f(rel) + "\n")
    return "".join(lines)


def format_matrix(mean, err) -> str:
    rows, cols = len(mean), len(mean[0])
    lines = [_d(rows) + _d(cols) + "\n"]
    for i in range(rows):
        for j in range(cols):
            m, e = mean[i][j], err[i][j]
            rel = e / m if m != 0 else math.inf
            lines.append(_d(i) + _d(j) + _f(m) + _f(e) + _f(rel) + "\n")
    return "".join(lines)


def format_bins_scalar(bins) -> str:
    return _d(len(bins)) + "\n" + "".join(_d(b) + _f(v) + "\n" for b, v in enumerate(bins))


def format_bins_vector(bins) -> str:
    out = [_d(len(bins)) + _d(len(bins[0])) + "\n"]
    for b, row in enumerate(bins):
        out.extend(_d(b) + _d(i) + _f(v) + "\n" for i, v in enumerate(row))
    return "".join(out)


def format_bins_matrix(bins) -> str:
    out = [_d(len(bins)) + _d(len(bins[0])) + _d(len(bins[0][0])) + "\n"]
    for b, mat in enumerate(bins):
        for i, row in enumerate(mat):
            out.extend(_d(b) + _d(i) + _d(j) + _f(v) + "\n" for j, v in enumerate(row))
    return "".join(out)


def format_kstars(L: int, dim: int = 2) -> str:
    """DqmcIO::output_k_stars: the count, then 'index kx ky (kz)' per k star."""
    ks = kstars(L, dim)
    return _d(len(ks)) + "\n" + "".join(_d(i) + "".join(_f(c) for c in k) + "\n" for i, k in enumerate(ks))


def format_tgrids(beta: float, time_size: int) -> str:
    dt = beta / time_size
    return (_d(time_size) + _f(beta, 5) + _f(dt, 5) + "\n" +
            "".join(_d(t) + _f(t * dt) + "\n" for t in range(time_size)))


def format_fields(fields) -> str:
    """DqmcIO::output_bosonic_fields: 'Lt N' then 't i s' lines, fields[t][i] = +-1."""
    lt, n = len(fields), len(fields[0])
    out = [_d(lt) + _d(n) + "\n"]
    for t in range(lt):
        out.extend(_d(t) + _d(i) + _f(float(fields[t][i]), 1) + "\n" for i in range(n))
    return "".join(out)


def parse_fields(text: str):
    """DqmcIO::read_bosonic_fields_from_file: returns (Lt, N, fields[t][i] in {+1, -1})."""
    tok = text.split()
    lt, n = int(tok[0]), int(tok[1])
    f = [[1] * n for _ in range(lt)]
    vals = tok[2:]
    if len(vals) % 3:
        raise ValueError("fields file: expected 't i s' triples")
    for k in range(0, len(vals), 3):
        t, i, s = int(vals[k]), int(vals[k + 1]), float(vals[k + 2])
        if not (0 <= t < lt and 0 <= i < n):
            raise ValueError(f"fields file: site ({t}, {i}) outside {lt} x {n}")
        f[t][i] = 1 if s > 0 else -1
    return lt, n, f


def format_summary_line(description: str, mean: float, err: float) -> str:
    """DqmcIO::output_observable to the terminal: '%| 30s|%| 7s|%| 20.12f|  pm  %.12f'."""
    return f"{description:>30s}{'->':>7s}{mean:20.12f}  pm  {err:.12f}\n"


# the terminal descriptions (observable_handler.cpp:140-277) and the order in which
# dqmc_main prints the scalar results (src/dqmc_main.cpp:213-266)
DESCRIPTIONS = {
    "equaltime_sign": "Averaged sign (equal-time)", "dynamic_sign": "Averaged sign (dynamical)",
    "filling_number": "Filling number", "double_occupancy": "Double occupation", "kinetic_energy": "Kinetic energy",
    "local_spin_corr": "Local spin correlation", "momentum_distribution": "Momentum distribution",
    "spin_density_structure_factor": "SDW order parameter", "charge_density_structure_factor": "CDW order parameter",
    "s_wave_pairing_corr": "S-wave pairing correlation", "superfluid_stiffness": "Superfluid stiffness",
}
SUMMARY_SIGNS = ["equaltime_sign", "dynamic_sign"]
SUMMARY_ORDER = ["filling_number", "double_occupancy", "kinetic_energy", "local_spin_corr", "momentum_distribution",
                 "spin_density_structure_factor", "charge_density_structure_factor", "s_wave_pairing_corr",
                 "superfluid_stiffness"]


def format_summary(results: dict) -> str:
    """The scalar results as dqmc_main prints them: the two signs, a blank line, then the
    observables in the reference's fixed order (those measured)."""
    out = [format_summary_line(DESCRIPTIONS[n], *results[n]) for n in SUMMARY_SIGNS if n in results]
    out.append("\n")
    out += [format_summary_line(DESCRIPTIONS[n], *results[n]) for n in SUMMARY_ORDER if n in results]
    return "".join(out)


def _param(name: str, value: str) -> str:
    return f"{name:>30s}{'->':>7s}{value:>24s}\n"  # "%| 30s|%| 7s|%| 24s|\n"


def format_init_info(cfg: RunConfig, world_size: int) -> str:
    """DqmcIO::output_init_info (include/dqmc_io.h:101-236): model, lattice, checkerboard,
    Monte Carlo and measuring parameters.  world_size is the number of chains (the
    reference's MPI ranks); the bin count shown is bins per chain times chains."""
    f3 = lambda v: f"{v:.3f}"
    model = "Attractive Hubbard" if cfg.model == "AttractiveHubbard" else "Repulsive Hubbard"
    out = [f"   Model: {model}\n", _param("Hopping constant 't'", f3(cfg.hopping_t)),
           _param("Onsite interaction 'U'", f3(cfg.onsite_u)),
           _param("Checimcal potential 'mu'", f3(cfg.chemical_potential)), "\n"]  # the reference's spelling
    L, dim = cfg.L, cfg.dim
    ks = kstars(L, dim)
    k = ks[momentum_index(L, cfg.momentum, dim) if cfg.momentum else len(ks) - 1]
    if dim == 2:
        out += ["   Lattice: Square lattice\n", _param("Size of cell", f"{L} * {L}"),
                _param("Momentum point", f"({k[0] / math.pi:.2f}, {k[1] / math.pi:.2f}) pi")]
    else:
        out += ["   Lattice: Cubic lattice\n", _param("Size of cell", f"{L} * {L} * {L}"),
                _param("Momentum point", f"({k[0] / math.pi:.2f}, {k[1] / math.pi:.2f}, {k[2] / math.pi:.2f}) pi")]
    tf = lambda b: "True" if b else "False"
    out += [_param("Checkerboard breakups", tf(cfg.checkerboard)), "\n"]
    out += ["   MonteCarlo Params:\n", _param("Inverse temperature", f3(cfg.beta)),
            _param("Imaginary-time length", str(cfg.time_size)),
            _param("Imaginary-time interval", f3(cfg.beta / cfg.time_size)),
            _param("Stabilization pace", str(cfg.stabilization_pace)), "\n"]
    out += ["   Measuring Params:\n", _param("Warm up", tf(cfg.sweeps_warmup != 0)),
            _param("Equal-time measure", tf(bool(cfg.equaltime))), _param("Dynamical measure", tf(bool(cfg.dynamic))),
            "\n"]
    bins_per_chain = math.ceil(cfg.bin_num / world_size)
    out += [_param("Sweeps for warmup", str(cfg.sweeps_warmup)),
            _param("Number of bins", str(bins_per_chain * world_size)),
            _param("Sweeps per bin", str(cfg.bin_size)), _param("Sweeps between bins", str(cfg.sweeps_between_bins)),
            "\n"]
    return "".join(out)


def format_ending_info(seconds: float, wrap_error: float) -> str:
    """DqmcIO::output_ending_info (include/dqmc_io.h:241-265): wall time and the maximum
    wrapping error."""
    ms = int(seconds * 1000)  # Dqmc::timer() counts milliseconds
    day = ms // 86400000
    hour = int((ms / 1000 - day * 86400) // 3600)
    minute = int((ms / 1000 - day * 86400 - hour * 3600) // 60)
    sec = ms / 1000 - 86400 * day - 3600 * hour - 60 * minute
    if day:
        t = f"{day} d {hour} h {minute} m {sec:.2f} s"
    elif hour:
        t = f"{hour} h {minute} m {sec:.2f} s"
    elif minute:
        t = f"{minute} m {sec:.2f} s"
    else:
        t = f"{sec:.2f} s"
    return f"\n>> The simulation finished in {t}.\n\n>> Maximum of the wrapping error: {wrap_error:.5e}\n\n"


def analyse_bins(bins):
    """Observable::analyse (include/measure/observable.h:169-211): mean over bins and
    sqrt(<x^2> - <x>^2) / sqrt(nbins - 1), elementwise for vectors and matrices."""
    import numpy as np

    b = np.asarray(bins, dtype=np.float64)
    n = b.shape[0]
    mean = b.sum(axis=0) / n
    var = (b ** 2).sum(axis=0) / n - mean ** 2
    err = np.sqrt(np.maximum(var, 0.0)) / math.sqrt(n - 1) if n > 1 else np.zeros_like(mean)
    return mean, err
