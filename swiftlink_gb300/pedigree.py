"""Problem tables of a pedigree, built on the host without the reference.

`problem_from_workload(w)` turns a synthetic workload (`synth.make_workload`)
into the arrays `api.Problem.from_arrays` takes, in the reference's internal
conventions:

* members founders first, each group in pedigree-file order (Pedigree's
  internal order), mother/father -1 for founders;
* unphased genotype codes UNTYPED 0, HETERO 1, HOMOZ_A 2, HOMOZ_B 3 with
  allele "1" = A = the major allele (genotype.h:26-31,
  pedigree_parser.cc:39-64); a member is typed when any marker is
  (person.h:122-128);
* theta from the Haldane map function of the marker distances in Morgans and
  partial theta = haldane(inverse_haldane(theta) / (n + 1))
  (GeneticMap::sanity_check, genetic_map.cc:14-64; map_parser.cc:62);
* disease probabilities from the disease model (person.cc:85-119);
* the peel sequence from `sl_peel_sequence` (host code of the library);
* the non-ignorable meioses (markov_chain.cc:70-80 with
  Person::safe_to_ignore_meiosis, person.cc:208-222);
* the gene drop's own meiosis indicators as a legal starting graph `dg0`.
"""
from __future__ import annotations

import numpy as np

from swiftlink_gb300 import api
from swiftlink_gb300.workloads import disease_probs


def haldane(m):
    """GeneticMap::haldane (genetic_map.cc:84-86), m in Morgans."""
    return 0.5 * (1.0 - np.exp(-2.0 * m))


def inverse_haldane(r):
    """GeneticMap::inverse_haldane (genetic_map.cc:88-90)."""
    return -0.5 * np.log(1 - (2 * r))


def map_thetas(marker_cm, n_lod):
    g = np.asarray(marker_cm, np.float64) / 100.0
    theta = haldane(g[1:] - g[:-1])
    partial = haldane(inverse_haldane(theta) / float(n_lod + 1))
    return theta, partial


def meioses_of(mother, father, F):
    """Non-ignorable meioses: bit 2 (person - F) + parent, dropped when that
    parent is a founder with a single child."""
    N = len(mother)
    nchild = np.zeros(N, np.int64)
    for i in range(F, N):
        nchild[mother[i]] += 1
        nchild[father[i]] += 1
    out = []
    for b in range(2 * (N - F)):
        i, par = F + b // 2, b % 2
        parent = mother[i] if par == 0 else father[i]
        if not (parent < F and nchild[parent] == 1):
            out.append(b)
    return np.array(out or [0], np.int32)


def problem_from_workload(w, n_lod: int = 5) -> dict:
    persons = w.persons
    founders = [k for k, p in enumerate(persons) if p.founder]
    others = [k for k, p in enumerate(persons) if not p.founder]
    order = founders + others
    pos = {persons[k].pid: i for i, k in enumerate(order)}
    N, F, M = len(order), len(founders), w.marker_cm.size
    mother = np.full(N, -1, np.int32)
    father = np.full(N, -1, np.int32)
    sex = np.zeros(N, np.int32)
    affection = np.zeros(N, np.int32)
    geno = np.zeros((M, N), np.uint8)
    typed = np.zeros(N, np.uint8)
    dg0 = np.zeros((M, N, 2), np.int32)
    for i, k in enumerate(order):
        p = persons[k]
        if not p.founder:
            mother[i] = pos[p.mother]
            father[i] = pos[p.father]
            dg0[:, i, :] = w.truth[k]
        sex[i] = p.sex
        affection[i] = p.affection
        a, b = w.genotypes[k, :, 0], w.genotypes[k, :, 1]
        code = np.where((a == 0) | (b == 0), 0, np.where(a != b, 1, np.where(a == 1, 2, 3)))
        geno[:, i] = code
        typed[i] = 1 if (code != 0).any() else 0
    spec = w.spec
    theta, partial = map_thetas(w.marker_cm, n_lod)
    ot, op, cut, prev, ch = api.peel_sequence(mother, father)
    return {
        "N": N, "F": F, "M": M, "K": len(ot), "n_lod": n_lod,
        "mother": mother, "father": father, "sex": sex, "typed": typed, "genotypes": geno,
        "affection": affection, "freq": np.float64(spec.disease_freq),
        "penetrance": np.array(spec.penetrance, np.float64),
        "disease_prob": disease_probs(affection, mother < 0, spec.disease_freq, spec.penetrance),
        "theta": theta, "partial": partial, "minor": np.asarray(w.maf, np.float64),
        "op_type": ot, "op_peel": op, "op_cutset": cut, "op_prev": prev, "op_children": ch,
        "meioses": meioses_of(mother, father, F), "dg0": dg0,
    }
