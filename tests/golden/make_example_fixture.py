"""Generate tests/golden/example_8x8.json from the reference's shipped example run.

The reference ships one run (example/config.toml, example/log.out and
example/output/fields.out): attractive Hubbard, 8x8, U=4, mu=0, beta=8,
Lt=160, stabilization pace 10, dense exp(-dtau K), all observables, 10 MPI
ranks x 2 bins.  This script reads those files from a reference checkout and
writes a compact fixture:
  * the model/lattice/Monte-Carlo parameters of example/config.toml,
  * the final 160x64 Ising configuration of example/output/fields.out,
    packed 1 bit per site (t-major, bit set = +1),
  * the mean +/- error of every equal-time observable and the maximum wrap
    error printed in example/log.out,
  * the mean +/- error of the dynamic observables of example/output/dos.out,
    dss.out and greens.out at a few tau (and k stars).

Usage: python tests/golden/make_example_fixture.py <reference-checkout>
"""
import json
import os
import re
import sys

import numpy as np

LOG_KEYS = {
    "Averaged sign (equal-time)": "equaltime_sign",
    "Filling number": "filling_number",
    "Double occupation": "double_occupancy",
    "Kinetic energy": "kinetic_energy",
    "Local spin correlation": "local_spin_corr",
    "Momentum distribution": "momentum_distribution",
    "SDW order parameter": "spin_density_structure_factor",
    "CDW order parameter": "charge_density_structure_factor",
    "S-wave pairing correlation": "s_wave_pairing_corr",
}


def main(ref: str) -> None:
    with open(os.path.join(ref, "example", "output", "fields.out")) as f:
        lt, n = (int(x) for x in f.readline().split())
        fields = np.zeros((lt, n), dtype=np.int8)
        for line in f:
            parts = line.split()
            if len(parts) == 3:
                fields[int(parts[0]), int(parts[1])] = 1 if float(parts[2]) > 0 else -1
    assert (fields != 0).all()
    packed = np.packbits((fields.reshape(-1) > 0).astype(np.uint8)).tobytes().hex()

    observables = {}
    wrap = None
    with open(os.path.join(ref, "example", "log.out")) as f:
        for line in f:
            m = re.search(r"Maximum of the wrapping error:\s*([0-9.eE+-]+)", line)
            if m:
                wrap = float(m.group(1))
            for label, key in LOG_KEYS.items():
                m = re.match(r"\s*" + re.escape(label) + r"\s*->\s*([-0-9.eE+]+)\s+pm\s+([-0-9.eE+]+)", line)
                if m:
                    observables[key] = [float(m.group(1)), float(m.group(2))]

    def table(name, ncols):
        rows = {}
        with open(os.path.join(ref, "example", "output", name)) as f:
            f.readline()
            for line in f:
                p = line.split()
                if len(p) == ncols:
                    rows[tuple(int(x) for x in p[:ncols - 3])] = [float(p[-3]), float(p[-2])]
        return rows

    taus = [0, 1, 5, 20, 80, 140, 159]
    dos, dss, greens = table("dos.out", 4), table("dss.out", 4), table("greens.out", 5)
    dynamic = {
        "taus": taus,
        "density_of_states": [dos[(t,)] for t in taus],
        "dynamic_spin_susceptibility": [dss[(t,)] for t in taus],
        "greens_kstars": [0, 7, 14],
        "greens_functions": [[greens[(k, t)] for t in taus] for k in (0, 7, 14)],
    }

    fixture = {
        "source": "reference example run: example/config.toml, example/log.out:42-55, example/output/fields.out",
        "model": "attractive", "L": 8, "hopping_t": 1.0, "onsite_u": 4.0, "mu": 0.0,
        "beta": 8.0, "Lt": lt, "pace": 10, "checkerboard": False, "momentum": "MPoint",
        "N": n, "bins_total": 20, "ranks": 10,
        "fields_packed_hex": packed,
        "max_wrap_error": wrap,
        "observables": observables,
        "dynamic": dynamic,
    }
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "example_8x8.json")
    with open(out, "w") as f:
        json.dump(fixture, f, indent=1)
    print("wrote", out, "observables:", sorted(observables))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <reference-checkout>")
    main(sys.argv[1])
