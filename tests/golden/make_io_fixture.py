"""Generate tests/golden/io_formats.json from the reference's shipped example output.

Reads example/output/*.out of a reference checkout and records, per file, a
SHA-256 digest of the whole file and its first lines (the size header and the
first data rows).  The I/O tests rebuild kstars.out, tgrids.out and fields.out
from the example's parameters and field configuration and compare digests, and
re-format the recorded rows of the observable files field by field, so the
writers' formats are pinned to the reference's own files.

It also records three blocks of the example's terminal log (example/log.out): the
parameter block of DqmcIO::output_init_info, the ending info and the scalar summary,
which the tests rebuild from the example's configuration and logged numbers.

Usage: python tests/golden/make_io_fixture.py <reference-checkout>
"""
import hashlib
import json
import os
import sys

FILES = ["kstars.out", "tgrids.out", "fields.out", "dos.out", "dos.bins.out", "dss.out", "dss.bins.out",
         "greens.out", "greens.bins.out", "swave.out", "swave.bins.out"]


def main(ref: str) -> None:
    out = {"source": "reference example run: example/output/*.out", "files": {}}
    for name in FILES:
        path = os.path.join(ref, "example", "output", name)
        with open(path, "rb") as f:
            data = f.read()
        lines = data.decode().split("\n")
        out["files"][name] = {"sha256": hashlib.sha256(data).hexdigest(), "head": lines[:4],
                              "lines": len(lines)}
    with open(os.path.join(ref, "example", "log.out"), encoding="utf-8") as f:
        log = f.read().split("\n")
    start = next(i for i, l in enumerate(log) if l.startswith("   Model:"))
    stop = next(i for i, l in enumerate(log) if l.startswith(" Warming up"))
    fin = next(i for i, l in enumerate(log) if l.startswith(">> The simulation finished"))
    summ = next(i for i, l in enumerate(log) if "Averaged sign (equal-time)" in l)
    end = max(i for i, l in enumerate(log) if " pm " in l)
    out["log"] = {"source": "reference example run: example/log.out",
                  "init_info": "\n".join(log[start:stop]),
                  "ending_info": "\n".join(log[fin - 1:fin + 4]),
                  "summary": "\n".join(log[summ:end + 1]) + "\n"}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io_formats.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <reference-checkout>")
    main(sys.argv[1])
