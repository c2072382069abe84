"""Run a reference configuration on the GPU and write the reference's output files.

    python -m dqmc_gb300.run -c config.toml -o DIR [-f FIELDS] [--walkers W] [--seed S]
                             [--precision fp64|mixed] [--rng minstd|philox]

(-c/--config, -o/--output and -f/--fields are dqmc_main's options, src/dqmc_main.cpp:53-62;
the configuration may also be given as the first positional argument.)

Follows the reference's driver (src/dqmc_main.cpp, src/dqmc.cpp:48-158): each walker
is one of the reference's MPI ranks (one Markov chain); warm-up of
sweeps_warmup / 2 forth-and-back sweeps; then ceil(bin_num / W) bins per walker,
each bin_size / 2 forth-and-back sweeps with measurements (with dynamic
observables the forward half-sweep is sweep_for_dynamic_greens and the equal-time
measurement is taken on the backward one), the normalisation of
MeasureHandler::normalize_stats, and sweeps_between_bins / 2 unmeasured sweeps
between bins; the bins of all walkers are pooled (the reference's MPI gather) and
analysed as Observable::analyse.  Under torchrun every process runs W walkers on its
own GPU and rank 0 gathers the bins, analyses and writes (the reference's MPI
layout, include/utils/mpi.hpp:29-104).  Output: the terminal summary of the scalar
observables and fields.out, kstars.out, tgrids.out, swave(.bins).out,
dos(.bins).out, greens(.bins).out, dss(.bins).out in the reference's formats.  As
in dqmc_main (src/dqmc_main.cpp:280-283), the final fields of walker 0 go to the
input fields file when one was given (so the next run resumes from them), else
to fields.out in the output folder.
G(k, tau) covers the configured `momentum_list` (rows of greens.out in the
reference's k-star order).
"""
from __future__ import annotations

import argparse
import math
import os
import sys
import time

import numpy as np

from . import io as dio
from . import parallel

def run(cfg: dio.RunConfig, out_dir: str, walkers: int = 1, seed: int = 12345, fields_file: str | None = None,
        precision: str = "fp64", rng: str = "minstd", log=None) -> dict:
    """Run the configuration; returns {name: (mean, error)} and writes the output files
    (rank 0 of a torchrun launch; the other ranks return {})."""
    import dqmc_gb300 as dq

    log = log if log is not None else sys.stdout  # resolved per call, so redirections apply
    rank, size = parallel.init()
    t_start = time.perf_counter()
    if size > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    L, lt, dim = cfg.L, cfg.time_size, cfg.dim
    kidx = dio.momentum_index(L, cfg.momentum, dim) if cfg.momentum else -1
    model = dq.ATTRACTIVE if cfg.model == "AttractiveHubbard" else dq.REPULSIVE
    descs = [dq.WalkerDesc(model=model, L=L, t=cfg.hopping_t, U=cfg.onsite_u, mu=cfg.chemical_potential,
                           beta=cfg.beta, Lt=lt, pace=cfg.stabilization_pace, checkerboard=cfg.checkerboard,
                           momentum_index=kidx, lattice=dq.CUBIC if dim == 3 else dq.SQUARE,
                           seed=seed + rank * walkers + w) for w in range(walkers)]
    b = dq.Batch(descs, rng=dq.RNG_PHILOX if rng == "philox" else dq.RNG_MINSTD,
                 precision=dq.MIXED if precision == "mixed" else dq.FP64)
    if rank == 0:
        log.write(">> Configurations of the bosonic fields "
                  + ("read from the input config file.\n\n" if fields_file else "set to random.\n\n"))
        log.write(">> Initialization finished. \n\n>> The simulation is going to get started with parameters "
                  "shown below :\n\n")
        log.write(dio.format_init_info(cfg, walkers * size))
    try:
        if fields_file:
            with open(fields_file, encoding="utf-8") as f:
                flt, fn, fields = dio.parse_fields(f.read())
            if flt != lt or fn != L ** dim:
                raise ValueError("fields file size does not match the configuration")
            for w in range(walkers):
                b.set_fields(w, np.array(fields, dtype=np.int8))
        else:
            for w in range(walkers):
                b.fields_random(w)
        b.init_greens()
        for _ in range(cfg.sweeps_warmup // 2):
            b.sweep_0_to_beta()
            b.sweep_beta_to_0()
        eqt, dyn = bool(cfg.equaltime), bool(cfg.dynamic)
        taus = list(range(lt))
        nbins = math.ceil(cfg.bin_num / (walkers * size)) if (eqt or dyn) else 0
        eq_bins = [[] for _ in range(walkers)]
        dyn_bins = {k: [[] for _ in range(walkers)] for k in ("greens", "dos", "dss", "rho", "sign")}
        ks = dio.kstars(L, dim)
        klist = [ks[i] for i in dio.momentum_list_indices(L, cfg.momentum_list or "KstarsAll", dim)]
        if eqt and not dyn:  # equal-time only: bins normalised on the device, one copy out
            binned = b.measure_bins(nbins, max(cfg.bin_size, 2), cfg.sweeps_between_bins)
            for w in range(walkers):
                eq_bins[w].extend(binned[w])
            nbins = 0
        for _ in range(nbins):
            b.clear_observables()
            if dyn:
                b.clear_dynamic()
            sgn = np.zeros(walkers)
            for _ in range(cfg.bin_size // 2):
                if dyn:
                    b.sweep_dynamic(taus)
                    sgn += [b.config_sign(w) for w in range(walkers)]
                else:
                    b.sweep_0_to_beta(measure=eqt)
                b.sweep_beta_to_0(measure=eqt)
            if eqt:
                sums, counts = b.observables_all()
                for w in range(walkers):
                    eq_bins[w].append(dq.write_bin(sums[w], counts[w]))
            if dyn:
                for w in range(walkers):
                    _, cnt = b.dynamic(w)
                    g = b.dynamic_greens_k(w, klist)  # [k][tau]
                    dos, dss, rho = b.dynamic_obs(w)
                    ms = sgn[w] / max(cnt[0], 1)  # the dynamic sign, one count per dynamic sweep
                    norm = cnt * ms
                    dyn_bins["greens"][w].append(g / norm[None, :])
                    dyn_bins["dos"][w].append(dos / norm)
                    dyn_bins["dss"][w].append(dss / norm)
                    dyn_bins["rho"][w].append(rho.sum() / (cnt[0] * ms))
                    dyn_bins["sign"][w].append(abs(ms))
            for _ in range(cfg.sweeps_between_bins // 2):
                b.sweep_0_to_beta()
                b.sweep_beta_to_0()
        fields0 = b.fields(0)
        wrap = max(b.wrap_error(w) for w in range(walkers))
    finally:
        b.close()

    eq_local = np.array([bb for wb in eq_bins for bb in wb])
    dyn_local = {k: np.array([x for wb in v for x in wb]) for k, v in dyn_bins.items()}
    eq_all = parallel.gather_bins(eq_local) if eqt else None
    dyn_all = {k: parallel.gather_bins(v) for k, v in dyn_local.items()} if dyn else None
    wrap_all = parallel.gather_bins(np.array([wrap]))
    if rank != 0:
        return {}
    log.write(dio.format_ending_info(time.perf_counter() - t_start, float(np.max(wrap_all))))
    os.makedirs(out_dir, exist_ok=True)
    results = {}

    def write(name, text):
        with open(os.path.join(out_dir, name), "w", encoding="utf-8") as f:
            f.write(text)

    if eqt:
        pooled = eq_all
        mean, err = dio.analyse_bins(pooled)
        for i, name in enumerate(dq.OBS_NAMES):
            if name == "equaltime_sign" or name in cfg.equaltime:
                results[name] = (float(mean[i]), float(err[i]))
        if "s_wave_pairing_corr" in cfg.equaltime:
            i = dq.OBS_NAMES.index("s_wave_pairing_corr")
            write("swave.out", dio.format_scalar(mean[i], err[i]))
            write("swave.bins.out", dio.format_bins_scalar(pooled[:, i]))
    if dyn:
        pool = dyn_all
        results["dynamic_sign"] = tuple(float(x) for x in dio.analyse_bins(pool["sign"]))
        for name, key, fname in (("density_of_states", "dos", "dos"), ("dynamic_spin_susceptibility", "dss", "dss")):
            if name in cfg.dynamic:
                mean, err = dio.analyse_bins(pool[key])
                write(f"{fname}.out", dio.format_vector(mean, err))
                write(f"{fname}.bins.out", dio.format_bins_vector(pool[key]))
        if "greens_functions" in cfg.dynamic:
            mean, err = dio.analyse_bins(pool["greens"])
            write("greens.out", dio.format_matrix(mean, err))
            write("greens.bins.out", dio.format_bins_matrix(pool["greens"]))
        if "superfluid_stiffness" in cfg.dynamic:
            mean, err = dio.analyse_bins(pool["rho"])
            results["superfluid_stiffness"] = (float(mean), float(err))
    if fields_file:  # dqmc_main writes the final fields back over the input file
        with open(fields_file, "w", encoding="utf-8") as f:
            f.write(dio.format_fields(fields0))
    else:
        write("fields.out", dio.format_fields(fields0))
    write("kstars.out", dio.format_kstars(L, dim))
    write("tgrids.out", dio.format_tgrids(cfg.beta, lt))
    log.write(dio.format_summary(results))
    return results


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("config_file", nargs="?", help="configuration file (same as -c)")
    ap.add_argument("-c", "--config", default=None, help="path of the TOML configuration file")
    ap.add_argument("-o", "--output", "--out", dest="out", default="output",
                    help="folder for the measured results (created if missing)")
    ap.add_argument("-f", "--fields", default=None,
                    help="fields file to start from (the reference's format); the final fields are written back to it")
    ap.add_argument("--walkers", type=int, default=1)
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--rng", choices=["minstd", "philox"], default="minstd")
    a = ap.parse_args(argv)
    config = a.config or a.config_file
    if not config:
        ap.error("a configuration file is required (-c/--config)")
    cfg = dio.load_config(config)
    run(cfg, a.out, walkers=a.walkers, seed=a.seed, fields_file=a.fields, precision=a.precision, rng=a.rng)
    return 0


if __name__ == "__main__":
    sys.exit(main())
