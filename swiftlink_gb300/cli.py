"""The `swift_gb300` program: LINKAGE ped/map/dat in, the LOD table out.

    python -m swiftlink_gb300.cli -p fam.ped -m fam.map -d fam.dat [-o out] [-i N] [-b N] ...

runs swiftlink_gb300/_build/swift_gb300 (built by `build.build()`), the C++
front end over the library's C ABI with the reference program's options
(main.cc).  Helpers read what it writes: the LOD table (LinkageWriter::write,
linkage_writer.cc:14-89) and the problem tables of its --dumpproblem mode.
"""
from __future__ import annotations

import os
import sys

import numpy as np

from swiftlink_gb300 import build as _build


def path() -> str:
    """The program's path; raises if it has not been built."""
    if not os.path.exists(_build.CLI):
        raise RuntimeError(f"{_build.CLI} is missing: run swiftlink_gb300.build.build() first")
    return _build.CLI


_INT_KEYS = ("mother", "father", "sex", "affection", "typed", "genotypes", "op_type", "op_peel")


def read_dump(fname: str) -> list:
    """The families of a --dumpproblem file, each a dict of arrays: members in
    internal order, genotypes [M][N], disease_prob [N][4], theta, partial,
    minor, gpos (Morgans), model = (freq, pen HOMO_U, HETERO, HOMO_A)."""
    fams = []
    cur = None
    with open(fname) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "family":
                cur = {"id": t[1], "N": int(t[2]), "F": int(t[3]), "M": int(t[4])}
                fams.append(cur)
            elif t[0] == "ids":
                cur["ids"] = t[1:]
            elif t[0] in _INT_KEYS:
                cur[t[0]] = np.array([int(x) for x in t[1:]], np.int64)
            else:
                cur[t[0]] = np.array([float(x) for x in t[1:]], np.float64)
    for d in fams:
        d["genotypes"] = d["genotypes"].reshape(d["M"], d["N"])
        d["disease_prob"] = d["disease_prob"].reshape(d["N"], 4)
    return fams


def read_lod_table(fname: str) -> dict:
    """The LOD table: marker names with their positions (cM), and per LOD
    position its position (cM), the total LOD and the per-family LODs (empty
    for one family)."""
    markers, pos, total, per = [], [], [], []
    with open(fname) as f:
        head = f.readline().split()
        assert head == ["marker", "position", "lod"], head
        for line in f:
            t = line.rstrip("\n").split("\t")
            if t[0] == "-":
                pos.append(float(t[1]))
                total.append(float(t[2]))
                per.append([float(x) for x in t[3:]])
            else:
                markers.append((t[0], float(t[1])))
    return {"markers": markers, "position": np.array(pos), "lod": np.array(total),
            "per_family": np.array(per)}


def main(argv=None) -> None:
    exe = path()
    args = sys.argv[1:] if argv is None else list(argv)
    os.execv(exe, [exe] + args)


if __name__ == "__main__":
    main()
