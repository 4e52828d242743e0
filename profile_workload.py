"""A short, fixed workload for ncu captures of the library's kernels.

    python profile_workload.py [--workload cfg2|cfg5] [--iterations 2] [--repeat 1] [--chains C]
        [--lprob 0.5] [--adjoint 0] [--adjoint-form F] [--adjoint-variant V] [--graph] [--lod-kernel K]
        [--ls-specialised] [--ls-kernel K]

cfg2 is the 120-member, 2000-SNP pedigree (10 chains by default); cfg5 the
400-member, 10,000-SNP pedigree (32 chains by default).  It runs `iterations`
device-driven MCMC iterations of `chains` chains in the fast sampler mode
(`repeat` times, each call continuing the chains),
kernels launched one by one with per-class event marks (with --graph: as one
launch of the run graph, no marks), then one batched FP32 LOD scoring of every
chain (the first scoring also times the LOD kernel candidates unless
--lod-kernel forces one of SL_LOD_KERNEL_*; --ls-specialised runs the
L-sampler compiled for the pedigree, --ls-kernel K asks for SL_LS_KERNEL_K,
e.g. a fixed lane group), and, with --adjoint G, the trait-peel
adjoint of G graphs under the dominant model (0.01, 0.8, 0.9), q = 1e-3, in
the form --adjoint-form fixes (SL_ADJOINT_*; 0: chosen by timing; for the
compiled form, --adjoint-variant picks its variant).  It prints
the per-kernel-class event times of the sampling part and the adjoint's time.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from swiftlink_gb300 import api  # noqa: E402
from swiftlink_gb300.workloads import disease_probs, load_problem  # noqa: E402


def problem(name):
    if name == "cfg2":
        return load_problem("cfg2")
    from swiftlink_gb300 import pedigree, synth
    return pedigree.problem_from_workload(synth.make_workload(int(name[3:])))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cfg2", choices=["cfg2", "cfg5"])
    ap.add_argument("--iterations", type=int, default=2)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--chains", type=int, default=0)
    ap.add_argument("--lprob", type=float, default=0.5)
    ap.add_argument("--adjoint", type=int, default=0)
    ap.add_argument("--adjoint-form", type=int, default=0)
    ap.add_argument("--adjoint-variant", type=int, default=0)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--lod-kernel", type=int, default=api.SL_LOD_KERNEL_AUTO)
    ap.add_argument("--ls-specialised", action="store_true")
    ap.add_argument("--ls-kernel", type=int, default=-1)
    a = ap.parse_args(argv)
    d = problem(a.workload)
    C = a.chains or (10 if a.workload == "cfg2" else 32)
    prob = api.Problem.from_arrays(d, with_legal=False)
    with api.Context(prob, n_chains=C, lod_precision=api.SL_LOD_FP32_RESCALED,
                     sampler_precision=api.SL_SAMPLER_FAST, lod_flags=api.SL_LOD_ZERO_OK,
                     lod_kernel=a.lod_kernel,
                     ls_kernel=a.ls_kernel if a.ls_kernel >= 0 else
                     (api.SL_LS_KERNEL_SPECIALISED if a.ls_specialised else api.SL_LS_KERNEL_GENERIC)) as ctx:
        ctx.set_graphs(np.stack([d["dg0"]] * C))
        ctx.profile(not a.graph)
        for r in range(a.repeat):
            t = time.perf_counter()
            ctx.run(iterations=(r + 1) * a.iterations, first_iteration=r * a.iterations, burnin=0,
                    period=1 << 30, lprob=a.lprob, seed=a.seed)
            ctx.synchronize()
            print(f"{a.iterations} iterations of {C} chains: {time.perf_counter() - t:.3f} s wall")
        if not a.graph:
            names = ["L-sampler", "M-sampler", "LOD", "LOD merge", "other"]
            for k in range(5):
                ms, n = ctx.profile_read(k)
                print(f"{names[k]:10s} {ms:9.3f} ms over {n} marks")
            ctx.profile(False)
        ctx.lod_score_chains()
        ctx.synchronize()
        graphs = ctx.get_graphs()
        print("lod kernel", ctx.lod_kernel_info(), "ls lanes and tuning", ctx.ls_tuning())
    if a.adjoint > 0:
        pen, q = (0.01, 0.8, 0.9), 1e-3
        dd = dict(d, penetrance=np.array(pen), freq=np.float64(q),
                  disease_prob=disease_probs(d["affection"], d["mother"] < 0, q, pen))
        with api.Context(api.Problem.from_arrays(dd, with_legal=False), n_chains=1,
                         lod_precision=api.SL_LOD_FP32_RESCALED, lod_flags=api.SL_LOD_ZERO_OK) as actx:
            gset = np.stack([graphs[i % C] for i in range(a.adjoint)])
            actx.adjoint_set_form(a.adjoint_form, a.adjoint_variant)
            t = time.perf_counter()
            grad, pt = actx.trait_backward(gset)
            dt = time.perf_counter() - t
            print("adjoint", grad.shape, float(np.abs(grad).max()), pt)
            print(f"adjoint: {dt:.3f} s wall for the first call (compiles and timing included); form and timed "
                  f"launches (warp, thread, specialised ms): {actx.adjoint_info()}; specialised (shapes, variant, "
                  f"registers, compile ms): {actx.adjoint_kernel_info()}")
            t = time.perf_counter()
            actx.trait_backward(gset)
            dt = time.perf_counter() - t
            print(f"adjoint: second call {dt:.3f} s wall, {grad[..., 0].size / dt:.4g} positions/s")


if __name__ == "__main__":
    main()
