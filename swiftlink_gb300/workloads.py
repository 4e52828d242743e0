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


def disease_probs(affection, founder, freq, penetrance):
    """Person::disease_prob (person.cc:85-119) from the disease model
    (DiseaseModel::get_apriori_prob2 / get_penetrance_prob2,
    disease_model.cc:139-187), autosomal, phased order UU, AA, AU, UA.
    affection: 0 unknown, 1 unaffected, 2 affected; founder: bool per person."""
    affection = np.asarray(affection)
    founder = np.asarray(founder, bool)
    q = float(freq)
    pen = [float(x) for x in penetrance]
    prior = [(1.0 - q) * (1.0 - q), q * (1.0 - q), q * q]   # HOMO_U, HETERO, HOMO_A
    unph = [0, 2, 1, 1]                                     # UU, AA, AU, UA -> unphased trait
    out = np.zeros((affection.size, 4))
    for i, (a, f) in enumerate(zip(affection, founder)):
        for v in range(4):
            t = unph[v]
            if f:
                if a == 2:
                    out[i, v] = prior[t] * pen[t]
                elif a == 1:
                    out[i, v] = prior[t] * (1.0 - pen[t])
                else:
                    out[i, v] = (prior[t] * pen[t]) + (prior[t] * (1.0 - pen[t]))
            else:
                if a == 2:
                    out[i, v] = pen[t]
                elif a == 1:
                    out[i, v] = 1.0 - pen[t]
                else:
                    out[i, v] = 0.25
    return out
