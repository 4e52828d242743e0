"""Seeded synthetic LINKAGE workloads for the linkage MCMC hot path.

A workload is a consanguineous pedigree (founder couples, sibships, marry-in
spouses and first/second-cousin marriages that close loops), biallelic SNP
genotypes gene-dropped under the Haldane map, a disease locus placed between
markers, and affection statuses that are consistent with the disease model.
The output is the three LINKAGE files the `swift` program reads
(pedfile columns: famid id father mother sex affection a1 a2 ...,
pedigree_parser.cc:80-161; mapfile: chromosome, cM, name, map_parser.cc:20-62;
datfile: trait locus first, then one "3 2" numbered-allele block per SNP,
linkage_parser.cc:254-330).

No public dataset is involved: every workload is produced from a seed
(20261203 + config number by default) so the same files can be regenerated on
any machine.  Everything here is numpy on the host; nothing is timed.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

SEED_BASE = 20261203


@dataclasses.dataclass
class WorkloadSpec:
    """Shape of one synthetic linkage workload."""

    n_members: int
    generations: int
    loops: int
    affected: int
    markers: int
    spacing_cm: float
    maf: Tuple[float, float]
    missing_founders: float = 0.0
    missing_all: float = 0.0
    disease_cm: float = 50.0
    penetrance: Tuple[float, float, float] = (0.0, 0.0, 1.0)
    disease_freq: float = 1e-4
    n_founders: Optional[int] = None
    lod_per_interval: int = 5


# The five workloads the hot path is measured on.
CONFIGS: Dict[int, WorkloadSpec] = {
    # 30 members, 10 founders, 4 generations, one first-cousin loop,
    # 5 affected children; 200 SNPs at 0.5 cM; founders 10% missing.
    1: WorkloadSpec(n_members=30, n_founders=10, generations=4, loops=1, affected=5,
                    markers=200, spacing_cm=0.5, maf=(0.1, 0.5), missing_founders=0.10),
    # 120 members, 6 generations, 3 loops, 35 affected; 2000 SNPs at 0.2 cM, 5% MAR.
    2: WorkloadSpec(n_members=120, generations=6, loops=3, affected=35,
                    markers=2000, spacing_cm=0.2, maf=(0.05, 0.5), missing_all=0.05),
    # the config-2 pedigree under a dominant, incompletely penetrant model
    4: WorkloadSpec(n_members=120, generations=6, loops=3, affected=35,
                    markers=2000, spacing_cm=0.2, maf=(0.05, 0.5), missing_all=0.05,
                    penetrance=(0.01, 0.8, 0.9), disease_freq=1e-3),
    # 400 members, 8 generations, 10 loops, 60 affected; 10,000 SNPs at 0.1 cM.
    5: WorkloadSpec(n_members=400, generations=8, loops=10, affected=60,
                    markers=10000, spacing_cm=0.1, maf=(0.05, 0.5), missing_all=0.05),
}


def uneven_batch(n_pedigrees: int = 64, seed: int = SEED_BASE + 3, markers: int = 1000):
    """The uneven batch: `n_pedigrees` independent pedigrees with sizes drawn
    uniformly from 20-150 members and 0-4 loops, `markers` SNPs at 0.5 cM with
    MAF ~U(0.05, 0.5), the recessive model; each is a seeded workload (its own
    seed), built with the first shape that the topology builder accepts."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n_pedigrees:
        n = int(rng.integers(20, 151))
        loops = int(rng.integers(0, 5))
        gens = 3 + (n >= 40) + (n >= 90)
        loops = min(loops, max(0, gens - 3) * 2 + 1) if gens > 3 else min(loops, 1)
        spec = WorkloadSpec(n_members=n, generations=gens, loops=loops, affected=max(2, n // 10),
                            markers=markers, spacing_cm=0.5, maf=(0.05, 0.5), missing_all=0.02)
        try:
            out.append(make_workload(3, seed=int(rng.integers(1, 2**31)), spec=spec))
        except RuntimeError:
            continue
    return out


@dataclasses.dataclass
class Person:
    pid: int          # 1-based id written to the pedfile
    father: int       # 0 = unknown
    mother: int
    sex: int          # 1 male, 2 female
    gen: int
    affection: int = 1

    @property
    def founder(self) -> bool:
        return self.father == 0


@dataclasses.dataclass
class Workload:
    spec: WorkloadSpec
    persons: List[Person]
    marker_cm: np.ndarray        # [M] genetic positions in cM
    maf: np.ndarray              # [M] minor ("2") allele frequency
    genotypes: np.ndarray        # [N][M][2] alleles in {0,1,2} (0 = missing)
    truth: Optional[np.ndarray] = None   # [N][M][2] the meiosis indicators of the gene drop
    famid: str = "1"


def _ancestors(persons: Dict[int, Person], pid: int, depth: int) -> set:
    """Ancestors of pid up to `depth` generations back (excluding pid)."""
    out = set()
    frontier = {pid}
    for _ in range(depth):
        nxt = set()
        for q in frontier:
            p = persons[q]
            if not p.founder:
                nxt.add(p.father)
                nxt.add(p.mother)
        out |= nxt
        frontier = nxt
    return out


def _build_topology(rng: np.random.Generator, spec: WorkloadSpec) -> List[Person]:
    """Grow a pedigree generation by generation until it has spec.n_members.

    Generation 0 is a set of founder couples.  Each couple has 2-4 children;
    children of generation g (g < last) either marry a cousin (closing a loop),
    marry in a new founder, or stay single.  The last generation is trimmed so
    the member count is exact while every couple keeps at least one child.
    """
    target = spec.n_members
    G = spec.generations
    for attempt in range(2000):
        persons: Dict[int, Person] = {}
        nid = [0]

        def new(sex, father, mother, gen):
            nid[0] += 1
            persons[nid[0]] = Person(nid[0], father, mother, sex, gen)
            return nid[0]

        # expected growth: choose the number of founder couples and marry-in rate
        # a single founder couple keeps the pedigree one connected family
        n0 = 1
        couples = []
        for _ in range(n0):
            f = new(1, 0, 0, 0)
            m = new(2, 0, 0, 0)
            couples.append((f, m))
        loops_left = spec.loops
        # loops are closed in the generations that have cousins (g >= 2)
        loop_gens = list(range(2, G - 1)) or [G - 2]
        loops_per_gen = {g: 0 for g in loop_gens}
        for i in range(spec.loops):
            loops_per_gen[loop_gens[-1 - (i % len(loop_gens))]] += 1
        loop_couples = []
        ok = True
        for g in range(1, G):
            kids = []
            for (f, m) in couples:
                nk = int(rng.integers(2, 6))
                for _ in range(nk):
                    kids.append(new(int(rng.integers(1, 3)), f, m, g))
            if g == G - 1:
                break
            # marriages for the next generation
            single = list(kids)
            rng.shuffle(single)
            next_couples = []
            want_loops = loops_per_gen.get(g, 0)
            for _ in range(want_loops):
                found = None
                for i in range(len(single)):
                    a = persons[single[i]]
                    anc_a = _ancestors(persons, a.pid, 3)
                    for j in range(len(single)):
                        if i == j:
                            continue
                        b = persons[single[j]]
                        if a.sex == b.sex:
                            continue
                        if a.father == b.father:  # siblings
                            continue
                        if anc_a & _ancestors(persons, b.pid, 3):
                            found = (single[i], single[j])
                            break
                    if found:
                        break
                if not found:
                    ok = False
                    break
                a, b = found
                single.remove(a)
                single.remove(b)
                fa, mo = (a, b) if persons[a].sex == 1 else (b, a)
                next_couples.append((fa, mo))
                loop_couples.append((fa, mo))
                loops_left -= 1
            if not ok:
                break
            # growth control: generation sizes rise until the target is in reach
            remaining_gens = G - 1 - g
            size_now = len(persons)
            need = max(0, target - size_now)
            per_couple = 3.0 + 1.0  # children + marry-in spouse
            want_couples = int(np.ceil(need / (per_couple * max(1, remaining_gens)))) + 1
            want_couples = max(want_couples, 1)
            for pid in single:
                if len(next_couples) >= want_couples + want_loops:
                    break
                p = persons[pid]
                spouse = new(2 if p.sex == 1 else 1, 0, 0, g)
                next_couples.append((pid, spouse) if p.sex == 1 else (spouse, pid))
            couples = next_couples
        if not ok or loops_left:
            continue
        # trim / extend the last generation to hit the exact size
        last = [p.pid for p in persons.values() if p.gen == G - 1 and not p.founder]
        n = len(persons)
        if n < target:
            # extend: add children to last-generation couples
            for _ in range(target - n):
                f, m = couples[int(rng.integers(0, len(couples)))]
                new(int(rng.integers(1, 3)), f, m, G - 1)
        elif n > target:
            counts: Dict[Tuple[int, int], int] = {}
            for pid in last:
                p = persons[pid]
                counts[(p.father, p.mother)] = counts.get((p.father, p.mother), 0) + 1
            removable = [pid for pid in last]
            rng.shuffle(removable)
            excess = n - target
            removed = []
            for pid in removable:
                if excess == 0:
                    break
                p = persons[pid]
                key = (p.father, p.mother)
                if counts[key] > 1:
                    counts[key] -= 1
                    removed.append(pid)
                    excess -= 1
            if excess:
                continue
            for pid in removed:
                del persons[pid]
        if len(persons) != target:
            continue
        nf = sum(1 for p in persons.values() if p.founder)
        if spec.n_founders is not None and nf != spec.n_founders:
            continue
        # renumber 1..N in generation order, parents before children
        order = sorted(persons.values(), key=lambda p: (p.gen, p.pid))
        remap = {p.pid: i + 1 for i, p in enumerate(order)}
        out = []
        for p in order:
            out.append(Person(remap[p.pid], remap.get(p.father, 0), remap.get(p.mother, 0),
                              p.sex, p.gen))
        return out
    raise RuntimeError("could not build a pedigree with the requested shape")


def haldane(d_morgan: np.ndarray) -> np.ndarray:
    return 0.5 * (1.0 - np.exp(-2.0 * d_morgan))


def _gene_drop(rng, persons: List[Person], pos_cm: np.ndarray, founder_alleles):
    """Drop founder haplotypes down the pedigree along positions pos_cm.

    founder_alleles(pid) -> [2][L] allele array for a founder.  Returns
    {pid: [2][L]} with haplotype 0 maternal and 1 paternal.
    """
    theta = haldane(np.diff(pos_cm) / 100.0)
    hap = {}
    inherit = {}
    for p in persons:
        if p.founder:
            hap[p.pid] = founder_alleles(p.pid)
            continue
        kid = np.empty((2, pos_cm.size), dtype=np.int8)
        src_of = np.empty((2, pos_cm.size), dtype=np.int8)
        for slot, parent in ((0, p.mother), (1, p.father)):
            src = hap[parent]
            cross = rng.random(theta.size) < theta
            which = np.empty(pos_cm.size, dtype=np.int64)
            which[0] = rng.integers(0, 2)
            which[1:] = (which[0] + np.cumsum(cross)) % 2
            kid[slot] = src[which, np.arange(pos_cm.size)]
            src_of[slot] = which
        hap[p.pid] = kid
        inherit[p.pid] = src_of
    _gene_drop.inherit = inherit   # the true meiosis indicators of the last drop
    return hap


def make_workload(cfg: int = 1, seed: Optional[int] = None,
                  spec: Optional[WorkloadSpec] = None) -> Workload:
    """Build the seeded workload for config `cfg` (or an explicit spec)."""
    if spec is None:
        spec = CONFIGS[cfg]
    if seed is None:
        seed = SEED_BASE + cfg
    rng = np.random.default_rng(seed)
    persons = _build_topology(rng, spec)
    M = spec.markers
    marker_cm = spec.spacing_cm * (np.arange(M) + 0.5)
    maf = rng.uniform(spec.maf[0], spec.maf[1], size=M)
    # disease locus inserted between markers
    dpos = spec.disease_cm
    all_pos = np.sort(np.concatenate([marker_cm, [dpos]]))
    didx = int(np.searchsorted(all_pos, dpos))
    pen = spec.penetrance
    recessive = pen[0] == 0.0 and pen[1] == 0.0
    founders = [p.pid for p in persons if p.founder]
    target = spec.affected
    nonfounders = [p for p in persons if not p.founder]
    for attempt in range(400):
        carrier_rate = min(0.95, 0.25 + 0.02 * attempt) if recessive else min(0.6, 0.15 + 0.01 * attempt)

        def founder_alleles(pid, carrier_rate=carrier_rate):
            h = (rng.random((2, all_pos.size)) < np.concatenate([maf[:didx], [0.0], maf[didx:]])[None, :])
            h = h.astype(np.int8)
            h[:, didx] = (rng.random(2) < carrier_rate).astype(np.int8)
            return h

        hap = _gene_drop(rng, persons, all_pos, founder_alleles)
        dis = {pid: int(h[0, didx] + h[1, didx]) for pid, h in hap.items()}  # copies of disease allele
        if recessive:
            cand = [p.pid for p in nonfounders if dis[p.pid] == 2]
        else:
            cand = [p.pid for p in nonfounders if dis[p.pid] >= 1]
        if len(cand) < target:
            continue
        # prefer later generations
        gen_of = {p.pid: p.gen for p in persons}
        cand.sort(key=lambda q: (-gen_of[q], q))
        chosen = set(cand[:target])
        for p in persons:
            if p.pid in chosen:
                p.affection = 2
            elif recessive and dis[p.pid] == 2:
                p.affection = 0  # unknown: an unaffected homozygote is impossible under the model
            else:
                p.affection = 1
        break
    else:
        raise RuntimeError("could not place enough affected individuals")
    N = len(persons)
    geno = np.zeros((N, M, 2), dtype=np.int8)
    keep = np.ones(all_pos.size, dtype=bool)
    keep[didx] = False
    for i, p in enumerate(persons):
        h = hap[p.pid][:, keep]  # [2][M], 1 = minor allele
        geno[i, :, 0] = h[0] + 1
        geno[i, :, 1] = h[1] + 1
        miss_rate = spec.missing_all + (spec.missing_founders if p.founder else 0.0)
        if miss_rate > 0:
            miss = rng.random(M) < miss_rate
            geno[i, miss, :] = 0
    # the true descent graph at the markers: indicator 0 = the parent's maternal haplotype
    inherit = _gene_drop.inherit
    truth = np.zeros((N, M, 2), dtype=np.int8)
    for i, p in enumerate(persons):
        if not p.founder:
            truth[i] = inherit[p.pid][:, keep].T
    return Workload(spec=spec, persons=persons, marker_cm=marker_cm, maf=maf, genotypes=geno, truth=truth)


def write_linkage(w: Workload, prefix: str) -> Tuple[str, str, str]:
    """Write prefix.ped / prefix.map / prefix.dat and return the three paths."""
    d = os.path.dirname(prefix)
    if d:
        os.makedirs(d, exist_ok=True)
    ped, mapf, dat = prefix + ".ped", prefix + ".map", prefix + ".dat"
    M = w.marker_cm.size
    with open(ped, "w") as f:
        for i, p in enumerate(w.persons):
            g = w.genotypes[i].reshape(-1)
            f.write(f"{w.famid} {p.pid} {p.father} {p.mother} {p.sex} {p.affection} ")
            f.write(" ".join(str(int(x)) for x in g))
            f.write("\n")
    with open(mapf, "w") as f:
        f.write("#Chr Genpos Marker\n")
        for j in range(M):
            f.write(f"1 {w.marker_cm[j]:.6f} snp{j + 1}\n")
    s = w.spec
    with open(dat, "w") as f:
        f.write(f"{M + 1} 0 0 5\n")
        f.write("0 0.0 0.0 0\n")
        f.write(" ".join(str(i + 1) for i in range(M + 1)) + "\n")
        f.write("1 2 # TRAIT\n")
        f.write(f"{1.0 - s.disease_freq:.10g} {s.disease_freq:.10g}\n")
        f.write("1\n")
        f.write(f"{s.penetrance[0]:.6f} {s.penetrance[1]:.6f} {s.penetrance[2]:.6f}\n")
        for j in range(M):
            f.write(f"3 2 # snp{j + 1}\n")
            f.write(f"{1.0 - w.maf[j]:.10f} {w.maf[j]:.10f}\n")
        f.write("0 0\n")
        th = haldane(np.diff(w.marker_cm) / 100.0)
        f.write("0.1 " + " ".join(f"{t:.10g}" for t in th) + "\n")
        f.write("1 2.0 1.0\n")
    return ped, mapf, dat


def workload_files(cfg: int, outdir: str, seed: Optional[int] = None,
                   spec: Optional[WorkloadSpec] = None) -> Tuple[str, str, str]:
    """Generate config `cfg` into outdir (cached by name) and return the paths."""
    tag = f"cfg{cfg}" if seed is None and spec is None else f"cfg{cfg}_s{seed}"
    prefix = os.path.join(outdir, tag)
    paths = (prefix + ".ped", prefix + ".map", prefix + ".dat")
    if all(os.path.exists(p) for p in paths):
        return paths
    w = make_workload(cfg, seed=seed, spec=spec)
    return write_linkage(w, prefix)
