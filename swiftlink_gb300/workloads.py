"""Measured workloads: problem tables of a seeded synthetic pedigree.

`load_problem("cfg2")` returns the 120-member, 2000-SNP pedigree (3 loops,
35 affected, recessive model) with its peel sequence and a legal starting
descent graph, as written by tests/golden/make_golden.py from the seeded
generator in swiftlink_gb300/synth.py.
"""
from __future__ import annotations

import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _lists(off, flat):
    return [flat[off[i]:off[i + 1]].astype(np.int32) for i in range(len(off) - 1)]


def load_problem(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, f"{name}_problem.npz"))
    d = {k: z[k] for k in z.files}
    for k in ("op_cutset", "op_prev", "op_children"):
        d[k] = _lists(d.pop(k + "_off"), d.pop(k + "_flat"))
    for k in ("N", "F", "M", "K", "n_lod"):
        d[k] = int(d[k])
    n = d["M"] * d["N"] * 2
    d["dg0"] = np.unpackbits(d.pop("dg0_bits"))[:n].reshape(d["M"], d["N"], 2).astype(np.int32)
    return d


def step_bytes(N: int, F: int, M: int) -> int:
    """Algorithmic bytes of one descent-graph step: 2-bit genotypes, the
    bit-packed non-founder indicators read and written, and 8 bytes of map
    data per locus: M * (ceil(N/4) + 2*ceil(Nnf/4) + 8)."""
    nnf = N - F
    return M * (-(-N // 4) + 2 * (-(-nnf // 4)) + 8)


def position_bytes(N: int, F: int, n: int) -> float:
    """Algorithmic bytes of one LOD position: the two flanking indicator
    columns shared by the n positions of an interval, the partial theta, and
    the FP64 accumulator read-modify-write: (2*ceil(Nnf/4) + 4)/n + 16."""
    nnf = N - F
    return (2 * (-(-nnf // 4)) + 4) / n + 16
