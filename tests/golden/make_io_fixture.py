"""Generate tests/golden/io_formats.json from the reference's shipped example output.

Reads example/output/*.out of a reference checkout and records, per file, a
SHA-256 digest of the whole file and its first lines (the size header and the
first data rows).  The I/O tests rebuild kstars.out, tgrids.out and fields.out
from the example's parameters and field configuration and compare digests, and
re-format the recorded rows of the observable files field by field, so the
writers' formats are pinned to the reference's own files.

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
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io_formats.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
