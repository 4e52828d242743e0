"""Write the golden fixtures in tests/golden/ from the reference's own code.

Runs only where the reference sources exist (they are compiled into
oracle/_ref/libswiftref.so by `make -C oracle ref`).  For each case it stores
the problem exactly as the reference builds it (internal person order, peel
sequence, genotype-elimination masks, priors), a starting descent graph from
the reference's sequential imputation, and the reference's outputs for:

  * a chain of single-locus L-sampler steps with given uniforms,
  * an even-then-odd L-sweep with per-locus uniforms,
  * an M-sweep over a shuffled meiosis order with per-step uniforms,
  * LOD raw log-sums, count and P(T) for three descent graphs.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import dataclasses
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from swiftlink_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root():
    """The reference's root directory, as oracle/Makefile's REF names it."""
    out = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"], check=True,
                         capture_output=True, text=True).stdout.strip()
    return out


REF_EXAMPLES = os.path.join(reference_root(), "examples")
INPUTS = tempfile.mkdtemp(prefix="swiftlink_golden_")


def csr(lists):
    off = np.zeros(len(lists) + 1, np.int32)
    for i, x in enumerate(lists):
        off[i + 1] = off[i] + len(x)
    flat = np.concatenate([np.asarray(x, np.int32) for x in lists]) if off[-1] else np.zeros(0, np.int32)
    return off, flat.astype(np.int32)


def case_paths(name):
    if name in ("east", "loop"):
        return tuple(os.path.join(REF_EXAMPLES, f"{name}.{ext}") for ext in ("ped", "map", "dat"))
    cfg = int(name[3:])
    return synth.workload_files(cfg, INPUTS)


def make(name, seed):
    r = ref.Ref(*case_paths(name), n_lod=5, peel_iters=10000, seed=seed)
    p = r.problem()
    d = dataclasses.asdict(p)
    out = {k: v for k, v in d.items() if isinstance(v, np.ndarray)}
    for k in ("N", "F", "M", "K", "n_lod"):
        out[k] = np.int64(d[k])
    out["freq"] = np.float64(p.freq)
    for k in ("op_cutset", "op_prev", "op_children"):
        out[k + "_off"], out[k + "_flat"] = csr(d[k])
    rng = np.random.default_rng(seed)
    dg0, ll0 = r.initial_dg(si_iters=5)
    out["dg0"], out["loglik0"] = dg0, np.float64(ll0)
    stride = p.K + 2 * p.N
    # chain of single-locus steps
    loci = np.unique(np.concatenate([[0, p.M - 1, p.M // 2], rng.integers(0, p.M, 5)])).astype(np.int32)
    us = rng.random((loci.size, stride))
    dg = dg0.copy()
    after = []
    used = []
    for i, l in enumerate(loci):
        dg, n = r.lstep(dg, int(l), us[i])
        after.append(dg.copy())
        used.append(n)
    out["lstep_loci"], out["lstep_u"] = loci, us
    out["lstep_after"], out["lstep_used"] = np.stack(after), np.array(used, np.int32)
    # even-then-odd sweep, draws per locus
    usw = rng.random((p.M, stride))
    dg = dg0.copy()
    for l in list(range(0, p.M, 2)) + list(range(1, p.M, 2)):
        dg, _ = r.lstep(dg, l, usw[l])
    out["lsweep_u"], out["lsweep_after"] = usw, dg.copy()
    dg_l = dg.copy()
    # M-sweep
    order = p.meioses.copy()
    rng.shuffle(order)
    um = rng.random((order.size, p.M))
    dgm, mused = r.msweep(dg_l, order, um)
    out["msweep_order"], out["msweep_u"] = order.astype(np.int32), um
    out["msweep_after"], out["msweep_used"] = dgm, mused
    # LOD over three graphs
    graphs = np.stack([dg0, dg_l, dgm])
    raw, cnt, tp = r.lod(graphs)
    out["lod_graphs"], out["lod_raw"] = graphs, raw
    out["lod_count"], out["lod_trait_prob"] = np.int64(cnt), np.float64(tp)
    r.close()
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(name, path, os.path.getsize(path))


def make_problem_only(name, seed):
    """Problem tables plus one legal starting graph (bit-packed), no outputs:
    the seeded large-size cases whose expected values come from the C port."""
    r = ref.Ref(*case_paths(name), n_lod=5, peel_iters=10000, seed=seed)
    p = r.problem()
    d = dataclasses.asdict(p)
    out = {k: v for k, v in d.items() if isinstance(v, np.ndarray) and k != "trait_prior"}
    for k in ("N", "F", "M", "K", "n_lod"):
        out[k] = np.int64(d[k])
    out["freq"] = np.float64(p.freq)
    for k in ("op_cutset", "op_prev", "op_children"):
        out[k + "_off"], out[k + "_flat"] = csr(d[k])
    dg0, ll0 = r.initial_dg(si_iters=2)
    out["dg0_bits"] = np.packbits(dg0.astype(np.uint8).reshape(-1))
    out["loglik0"] = np.float64(ll0)
    r.close()
    path = os.path.join(HERE, f"{name}_problem.npz")
    np.savez_compressed(path, **out)
    print(name, path, os.path.getsize(path))


if __name__ == "__main__":
    if not ref.available():
        sys.exit("reference build missing: run `make -C oracle ref` first")
    for name, seed in (("loop", 11), ("east", 12), ("cfg1", 13)):
        make(name, seed)
    make_problem_only("cfg2", 14)
