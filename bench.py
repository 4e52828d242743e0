#!/usr/bin/env python
"""Benchmark of the SwiftLink MCMC hot path on GB300.

Workload: the seeded synthetic 120-member, 6-generation pedigree with 3
consanguinity loops and 35 affected, 2,000 SNPs at 0.2 cM, recessive model,
10 replicate chains per GPU, scoring every 100th descent graph at 5 positions
per marker interval (9,995 LOD positions per scored graph).

A step is one MCMC iteration (MarkovChain::run, markov_chain.cc:335-392) of
every chain: an L-sweep over all 2,000 loci or an M-sweep over all 184
non-ignorable meioses, chosen per chain with probability 0.5, plus LOD scoring
on iterations that are multiples of 100.  `value` is descent-graph steps/s
over all chains and GPUs (batched form: all chains in each launch, FP32
rescaled LOD); LOD positions/s and the plain single-chain FP64 form are
reported beside it.

Arms:
  python bench.py [--gpus N --steps K --warmup W]           this implementation
  python bench.py --impl reference ...                        the reference's CPU
      path on the host cores (the C restatement in oracle/, one process per
      core, the reference's own build being unavailable on this machine)
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "descent-graph steps/s + LOD positions/s, batched vs plain GB300, |ΔLOD|≤1e-3"
UNIT = "steps/s"
CHAINS = 10
PERIOD = 100
STEP_ITERS = PERIOD   # MCMC iterations per timed step: one scoring period
LPROB = 0.5
SEED = 20261205
WORKLOAD = "cfg2"
L2_FLUSH_BYTES = 256 << 20  # larger than the 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--skip-uneven", action="store_true", help="leave out the uneven multi-pedigree batch")
    ap.add_argument("--skip-large", action="store_true", help="leave out the 400-member, 10,000-SNP workload")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def rank_max(x, dist=None, device="cpu"):
    """The maximum of x over the ranks of the process group (x itself without
    one): the timed region's length is the slowest rank's."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def config(world):
    return {"workload": "120-member 6-generation pedigree, 3 loops, 35 affected, 2000 SNPs at 0.2 cM, "
                        "recessive (0,0,1) q=1e-4, 10 replicate chains per GPU, scoring every 100th graph, "
                        "5 LOD positions per interval",
            "members": 120, "markers": 2000, "chains_per_gpu": CHAINS, "scoring_period": PERIOD,
            "lod_positions_per_graph": 9995, "lsampler_prob": LPROB,
            "parallelism": f"replicas x{world}",
            "step": "one scoring period: 100 MCMC iterations of every chain and one LOD scoring of every "
                    "chain's graph, one run-graph launch; value = chain-iterations/s",
            "l2": "flushed (256 MB write) before every timed step",
            "zero_likelihood_positions": "counted as zero terms of the log-sum (SL_LOD_ZERO_OK); the "
                                         "reference exits at the first one (peeler.cc:89-92)"}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the C restatement of the reference (oracle/)
# ---------------------------------------------------------------------------
def port_problem():
    from oracle import port
    from swiftlink_gb300.workloads import load_problem
    d = load_problem(WORKLOAD)
    d["trait_prior"] = port.derive_priors(d["genotypes"], d["typed"], d["minor"])
    return d


def port_iteration(P, d, dg, chain, it):
    """One MarkovChain::run iteration of one chain on the CPU port with the
    same Philox draw streams the device driver uses."""
    from swiftlink_gb300 import philox
    M, K, N = d["M"], d["K"], d["N"]
    if philox.chooses_l(SEED, chain, it, LPROB):
        u = philox.lsweep_draws(SEED, chain, it, M, K + 2 * N)
        for l in list(range(0, M, 2)) + list(range(1, M, 2)):
            dg, _ = P.lstep(dg, l, u[l])
    else:
        order = philox.shuffled(SEED, chain, it, d["meioses"])
        u = philox.msweep_draws(SEED, chain, it, order.size, M)
        dg, _ = P.msweep(dg, order, u)
    return dg


def cpu_baseline_sample():
    """~10-30 s of single-core CPU work: one L-sweep, one M-sweep and one LOD
    scoring of one chain, from which steps/s and positions/s follow."""
    from oracle import port
    port.build()
    d = port_problem()
    P = port.Port(d)
    M, K, N = d["M"], d["K"], d["N"]
    rng = np.random.default_rng(1)
    dg = d["dg0"].copy()
    t0 = time.perf_counter()
    u = rng.random((M, K + 2 * N))
    for l in list(range(0, M, 2)) + list(range(1, M, 2)):
        dg, _ = P.lstep(dg, l, u[l])
    tl = time.perf_counter() - t0
    order = d["meioses"].copy()
    rng.shuffle(order)
    t0 = time.perf_counter()
    dg, _ = P.msweep(dg, order, rng.random((order.size, M)))
    tm = time.perf_counter() - t0
    t0 = time.perf_counter()
    P.lod(dg[None], zero_ok=True)
    tlod = time.perf_counter() - t0
    steps_per_s = 2.0 / (tl + tm)
    return {"value": steps_per_s, "unit": UNIT, "cores": 1, "kind": "port",
            "lod_positions_per_s": (M - 1) * d["n_lod"] / tlod,
            "sample": f"one chain: 1 L-sweep ({tl:.2f} s) + 1 M-sweep over {order.size} meioses ({tm:.2f} s) "
                      f"+ 1 LOD scoring of 9995 positions ({tlod:.2f} s), single thread"}


def _ref_worker(args):
    chains, steps, warmup, budget_s = args
    from oracle import port
    d = port_problem()
    P = port.Port(d)
    dgs = {c: d["dg0"].copy() for c in chains}
    for it in range(warmup):
        for c in chains:
            dgs[c] = port_iteration(P, d, dgs[c], c, it)
    t0 = time.perf_counter()
    done = 0
    scored = 0
    for it in range(warmup, warmup + steps):
        for c in chains:
            dgs[c] = port_iteration(P, d, dgs[c], c, it)
        if it % PERIOD == 0:
            P.lod(np.stack([dgs[c] for c in chains]), zero_ok=True)
            scored += len(chains)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return done * len(chains), time.perf_counter() - t0, scored


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import port
    port.build()
    cores = os.cpu_count() or 1
    workers = max(1, min(cores, CHAINS * args.gpus))
    total_chains = CHAINS * args.gpus
    groups = [list(range(w, total_chains, workers)) for w in range(workers)]
    budget = 60.0
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(workers) as pool:
        res = pool.map(_ref_worker, [(g, args.steps, args.warmup, budget) for g in groups])
    wall = time.perf_counter() - t0
    chain_steps = sum(r[0] for r in res)
    tmax = max(r[1] for r in res)
    value = chain_steps / tmax
    min_steps = min(r[0] // max(1, len(g)) for r, g in zip(res, groups))
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tmax / max(1, min_steps),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded generator, swiftlink_gb300/synth.py)", "config": config(args.gpus),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                            "sample": f"C restatement of the reference, {workers} processes over "
                                      f"{total_chains} chains, {min_steps} timed iterations per chain "
                                      f"(capped at {budget:.0f} s), wall {wall:.1f} s"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# this implementation
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    from swiftlink_gb300 import api, philox
    from swiftlink_gb300.workloads import load_problem, step_bytes, position_bytes

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if dist:
            dist.barrier()

    def allmax(x):
        return rank_max(x, dist, dev)

    d = load_problem(WORKLOAD)
    prob = api.Problem.from_arrays(d, with_legal=False)
    N, F, M, n = d["N"], d["F"], d["M"], d["n_lod"]
    npos = (M - 1) * n
    C = CHAINS
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    seed = SEED + 7919 * rank

    # ---------------- batched form: all chains per launch, FP32-rescaled LOD
    # the L-sampler compiled for this pedigree (bit-identical to the generic kernel)
    ctx = api.Context(prob, n_chains=C, lod_precision=api.SL_LOD_FP32_RESCALED, device=local,
                      sampler_precision=api.SL_SAMPLER_FAST, lod_flags=api.SL_LOD_ZERO_OK,
                      ls_kernel=api.SL_LS_KERNEL_SPECIALISED)
    ls_sel, ls_ms = ctx.ls_kernel_info()
    ctx.set_graphs(np.stack([d["dg0"]] * C))
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    W, K = args.warmup, args.steps
    P_ = STEP_ITERS
    ctx.run(iterations=W * P_, burnin=0, period=PERIOD, lprob=LPROB, seed=seed)
    ctx.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = Clocks(local)
    launches0 = ctx.launches
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    # each step is one launch of the run graph: one scoring period, 100 MCMC
    # iterations of every chain (each chain running its own iterations) and the
    # scoring of every chain's graph at the period's first iteration
    for i in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xff)
            ev[i][0].record(stream)
        ctx.run(iterations=(W + i + 1) * P_, burnin=0, period=PERIOD, lprob=LPROB, seed=seed,
                first_iteration=(W + i) * P_)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    gpu_launches = ctx.launches - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_s = allmax(sum(step_ms) / 1e3)
    value = K * P_ * C * world / t_s

    # the same chains with one launch per MCMC iteration (every chain waits for
    # the slowest one at every iteration), for comparison
    Ki = min(K, 50)
    evi = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(Ki)]
    it0 = (W + K) * P_
    for i in range(Ki):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xff)
            evi[i][0].record(stream)
        ctx.run(iterations=it0 + i + 1, burnin=0, period=PERIOD, lprob=LPROB, seed=seed, first_iteration=it0 + i)
        with torch.cuda.stream(stream):
            evi[i][1].record(stream)
    ctx.synchronize()
    per_iter = {"value": Ki * C * world / allmax(sum(a.elapsed_time(b) for a, b in evi) / 1e3), "unit": UNIT,
                "note": "one run-graph launch (and L2 flush) per MCMC iteration: every chain waits for the "
                        "slowest at every iteration"}

    # algorithmic bytes of the timed run-graph launches: every chain-step moves
    # step_bytes, every scored graph position_bytes per position
    sb = step_bytes(N, F, M)
    scorings = K * P_ // PERIOD
    alg_total = K * P_ * C * sb + scorings * C * npos * position_bytes(N, F, n)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    per_launch = alg_total / K
    avg_s = sum(step_ms) / 1e3 / K
    achieved = per_launch / avg_s / 1e9
    run_graph_name = "run graph (one scoring period: 100 MCMC iterations of every chain)"
    # DRAM bytes per launch: the captured 2-iteration graph launch (per iteration in
    # profiles/traffic.md) times the iterations of one launch, an upper estimate (a
    # longer launch keeps more of its state in L2 between iterations)
    t_iter = traffic_from_profiles("run graph (one MCMC iteration of every chain)")
    traffic = t_iter * P_ if t_iter is not None else None

    # kernel shares from a separate profiled pass: the same iterations with
    # per-kernel-class events (the host-driven path, kernels launched one by one)
    lod_kernel_names = {api.SL_LOD_KERNEL_INTERP: "lod_prog_kernel", api.SL_LOD_KERNEL_JIT_REG: "sl_lod_jit (registers)",
                        api.SL_LOD_KERNEL_JIT_SMEM: "sl_lod_jit (shared memory)"}
    sel, jit_ms = ctx.lod_kernel_info()
    ls_name = "sl_ls_jit (specialised)" if ls_sel == api.SL_LS_KERNEL_SPECIALISED else "lsampler_kernel<float>"
    names = {0: ls_name, 1: "fag_warp_kernel+ffbs_scan_kernel", 2: lod_kernel_names.get(sel, "lod_kernel"),
             3: "lod_merge_kernel", 4: "choose/shuffle"}
    Kp = min(K, 10)
    ctx.profile(True)
    ctx.run(iterations=it0 + Ki + Kp, burnin=0, period=PERIOD, lprob=LPROB, seed=seed, first_iteration=it0 + Ki)
    ctx.synchronize()
    kern = {k: ctx.profile_read(k) for k in range(5)}
    ctx.profile(False)
    tot = max(1e-9, sum(x[0] for x in kern.values()))
    roofline = {"bound": "hbm", "kernel": run_graph_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "traffic_source": "profiles/traffic.md: ncu DRAM bytes of the run graph per iteration x 100",
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "when" in peaks else "fallback",
                "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": 1e3 * avg_s,
                "note": "latency-bound integer and FP32 work on small rfunctions: the HBM fraction is small by "
                        "construction; SM issue utilisation per kernel is in profiles/",
                "kernel_share_profiled_pass": {names[k]: round(v[0] / tot, 4) for k, v in kern.items()}}
    if WORKLOAD == "cfg2" and C == 10 and ls_sel == api.SL_LS_KERNEL_SPECIALISED:
        try:
            roofline["issue"] = issue_estimate(C, W * P_, (W + K) * P_, seed, LPROB, len(d["meioses"]),
                                               (clk or {}).get("sm_mhz"), torch.cuda.get_device_properties(dev).multi_processor_count,
                                               sum(step_ms) / 1e3)
        except Exception as exc:   # an estimate only: never lose the bench line over it
            roofline["issue"] = {"error": str(exc)[:200]}

    # ---------------- LOD positions/s, batched (many graphs per launch, FP32) vs plain (FP64, one graph)
    graphs = ctx.get_graphs()
    G = 64
    gset = np.stack([graphs[i % C] for i in range(G)])
    lctx = api.Context(prob, n_chains=G, lod_precision=api.SL_LOD_FP32_RESCALED, device=local, lod_flags=api.SL_LOD_ZERO_OK)
    lctx.set_graphs(gset)
    lstream = torch.cuda.ExternalStream(lctx.stream_handle())
    lod_pos_s = timed_lod(lctx, lstream, flush, G, npos, reps=5)
    lsel, ljit_ms = lctx.lod_kernel_info()
    pctx = api.Context(prob, n_chains=1, lod_precision=api.SL_LOD_FP64, device=local, lod_flags=api.SL_LOD_ZERO_OK)
    pctx.set_graphs(gset[:1])
    pstream = torch.cuda.ExternalStream(pctx.stream_handle())
    plain_lod_pos_s = timed_lod(pctx, pstream, flush, 1, npos, reps=3)

    # ---------------- the error of the batched form: one scoring of the 64-graph set in
    # FP32 with rescaling against FP64, per-position |dLOD|
    lctx.lod_reset()
    lctx.lod_score_chains()
    raw32, c32, tp32 = lctx.lod_results()
    with api.Context(prob, n_chains=G, lod_precision=api.SL_LOD_FP64, device=local,
                     lod_flags=api.SL_LOD_ZERO_OK) as p64:
        p64.set_graphs(gset)
        p64.lod_score_chains()
        raw64, c64, tp64 = p64.lod_results()
    fin = raw64 > -1e300
    dlod = float(np.abs(api.lod_table(raw32, c32, tp32) - api.lod_table(raw64, c64, tp64))[fin].max())

    # ---------------- adjoint of the trait peel (dominant model 0.01/0.8/0.9, q = 1e-3) over
    # the 64 stored graphs, through sl_trait_backward with host graphs and gradients
    adj = adjoint_rate(d, gset, local)

    # ---------------- the uneven batch: 64 pedigrees of 20-150 members, 8 MC3 chains each
    uneven = uneven_batch_rate(local) if not args.skip_uneven else None
    # ---------------- large scale: 400 members, 10,000 SNPs, 32 chains
    large = large_scale(local) if not args.skip_large else None

    # ---------------- plain form: one chain, FP64 LOD
    pctx.run(iterations=W, burnin=0, period=PERIOD, lprob=LPROB, seed=seed)
    pctx.synchronize()
    Kp = min(K, 40)
    evp = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(Kp)]
    for i in range(Kp):
        with torch.cuda.stream(pstream):
            flush.fill_(i & 0xff)
            evp[i][0].record(pstream)
        pctx.run(iterations=W + i + 1, burnin=0, period=PERIOD, lprob=LPROB, seed=seed, first_iteration=W + i)
        with torch.cuda.stream(pstream):
            evp[i][1].record(pstream)
    pctx.synchronize()
    plain_steps_s = Kp / (sum(a.elapsed_time(b) for a, b in evp) / 1e3)

    # ---------------- end to end through the public API with host buffers
    ectx = api.Context(prob, n_chains=C, lod_precision=api.SL_LOD_FP32_RESCALED, device=local,
                       sampler_precision=api.SL_SAMPLER_FAST, lod_flags=api.SL_LOD_ZERO_OK,
                       ls_kernel=api.SL_LS_KERNEL_SPECIALISED)
    host_graphs = np.ascontiguousarray(np.stack([d["dg0"]] * C))
    ectx.set_graphs(host_graphs)
    ectx.run(iterations=W * P_, burnin=0, period=PERIOD, lprob=LPROB, seed=seed)
    ectx.synchronize()
    host_graphs = ectx.get_graphs()
    Ke = min(K, 20)
    barrier()
    t0 = time.perf_counter()
    for i in range(Ke):
        ectx.set_graphs(host_graphs)                                   # H2D: the step's state
        ectx.run(iterations=(W + i + 1) * P_, burnin=0, period=PERIOD, lprob=LPROB, seed=seed,
                 first_iteration=(W + i) * P_)
        host_graphs = ectx.get_graphs()                                # D2H: the step's result
    e2e_t = allmax(time.perf_counter() - t0)
    words = M * ((2 * (N - F) + 31) // 32)
    e2e = {"value": Ke * P_ * C * world / e2e_t, "unit": UNIT, "h2d_bytes_per_step": 4 * words * C,
           "d2h_bytes_per_step": 4 * words * C,
           "path": "sl_set_descent_graphs (pinned, packed) + sl_run(one scoring period, 100 iterations) + "
                   "sl_get_descent_graphs per step"}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": t_s * 1e3 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64 peel and founder-allele graphs, f32 M-sampler filter, f32-rescaled LOD peel with "
                        "f64 accumulation (plain form: f64 throughout, bit-exact)",
               "data": "synthetic (seeded generator, swiftlink_gb300/synth.py; no public dataset)",
               "config": config(world), "impl": "ours",
               "lod_positions_per_s": lod_pos_s * world,
               "lod_kernel": {"selected": lod_kernel_names.get(lsel, str(lsel)),
                              "specialised_compile_ms": round(ljit_ms, 1),
                              "selection": "timed at the first scoring (SL_LOD_KERNEL_AUTO)"},
               "ls_kernel": {"selected": ls_name, "specialised_compile_ms": round(ls_ms, 1),
                             "selection": "SL_LS_KERNEL_SPECIALISED (NVRTC at context creation, outside the timed "
                                          "region; draws bit-identical graphs to the generic kernel)"},
               "plain": {"steps_per_s": plain_steps_s * world, "lod_positions_per_s": plain_lod_pos_s * world,
                         "form": "one chain per launch, exact FP64 samplers, FP64 LOD peel"},
               "batched_vs_plain": {"steps": value / (plain_steps_s * world),
                                    "lod_positions": lod_pos_s / plain_lod_pos_s},
               "max_abs_dlod_fp32_vs_fp64": dlod,
               "adjoint": adj,
               "uneven_batch": uneven,
               "large_scale": large,
               "per_iteration_launches": per_iter,
               "gpu_launches": int(gpu_launches), "roofline": roofline, "clocks": clk, "e2e": e2e}
        if world == 1:
            out["cpu_baseline"] = cpu_baseline_sample()
        print(json.dumps(out))
    for c in (ctx, lctx, pctx, ectx):
        c.close()
    if dist:
        dist.destroy_process_group()


def large_scale(device, C=32, K=4):
    """The 400-member, 8-generation, 10-loop pedigree with 10,000 SNPs at 0.1 cM
    (seeded, host-built peel sequence, the gene drop's graph as the start), 32
    chains: steps/s of the batched form (wall clock around sl_run of K
    iterations, one run-graph launch), LOD positions/s of the batched FP32 form
    against the plain FP64 form on the chains' 32 graphs, and the FP32 form's
    max |dLOD| against the FP64 peel with rescaling.  The plain FP64 peel (the
    reference's arithmetic) underflows to 0 at every position of this
    pedigree, so the rescaled FP64 peel is the accuracy yardstick."""
    from swiftlink_gb300 import api, pedigree, synth
    t0 = time.perf_counter()
    d = pedigree.problem_from_workload(synth.make_workload(5))
    prob = api.Problem.from_arrays(d, with_legal=False)
    ctx = api.Context(prob, n_chains=C, device=device, lod_precision=api.SL_LOD_FP32_RESCALED,
                      sampler_precision=api.SL_SAMPLER_FAST, lod_flags=api.SL_LOD_ZERO_OK,
                      ls_kernel=api.SL_LS_KERNEL_SPECIALISED)
    ctx.set_graphs(np.stack([d["dg0"]] * C))
    ctx.run(iterations=2, burnin=0, period=1, lprob=LPROB, seed=SEED)
    ctx.synchronize()
    setup_s = time.perf_counter() - t0
    t = time.perf_counter()
    ctx.run(iterations=2 + K, burnin=0, period=1 << 30, lprob=LPROB, seed=SEED, first_iteration=2)
    ctx.synchronize()
    steps_s = K * C / (time.perf_counter() - t)
    npos = (d["M"] - 1) * d["n_lod"]

    def lod_rate(c, reps):
        c.lod_score_chains()
        c.synchronize()
        c.lod_reset()
        t = time.perf_counter()
        for _ in range(reps):
            c.lod_score_chains()
        c.synchronize()
        return reps * C * npos / (time.perf_counter() - t)

    graphs = ctx.get_graphs()
    fp32 = lod_rate(ctx, 3)
    ctx.lod_reset()
    ctx.lod_score_chains()
    raw32, c32, tp32 = ctx.lod_results()
    out = {"members": d["N"], "founders": d["F"], "markers": d["M"], "chains": C, "steps_per_s": steps_s,
           "lod_positions_per_s": fp32, "setup_s": round(setup_s, 1),
           "max_cutset": int(max(len(c) for c in d["op_cutset"]))}
    for name, prec in (("plain_fp64", api.SL_LOD_FP64), ("fp64_rescaled", api.SL_LOD_FP64_RESCALED)):
        with api.Context(prob, n_chains=C, device=device, lod_precision=prec, lod_flags=api.SL_LOD_ZERO_OK) as c64:
            c64.set_graphs(graphs)
            rate = lod_rate(c64, 1)
            c64.lod_reset()
            c64.lod_score_chains()
            raw64, c_64, tp64 = c64.lod_results()
        fin = raw64 > -1e300
        out[name] = {"lod_positions_per_s": rate, "positions_underflowed": int((~fin).sum()),
                     "max_abs_dlod_fp32": float(np.abs(api.lod_table(raw32, c32, tp32)
                                                       - api.lod_table(raw64, c_64, tp64))[fin].max())
                     if fin.any() else None}
    out["batched_vs_plain_lod"] = fp32 / out["plain_fp64"]["lod_positions_per_s"]
    ctx.close()
    return out


def uneven_batch_rate(device, n_ped=64, chains=8, K=20):
    """Chain-steps/s of the uneven batch: 64 seeded pedigrees of 20-150
    members (0-4 loops, 1,000 SNPs at 0.5 cM), 8 MC3 chains each at
    temperatures 0.3^(j/7), fast samplers, FP32 LOD (the slot-program
    interpreter: no per-pedigree compilation), exchange and scoring every 10
    iterations, all pedigrees in one graph launch per spurt."""
    from swiftlink_gb300 import api, pedigree, synth
    t0 = time.perf_counter()
    probs = [pedigree.problem_from_workload(w) for w in synth.uneven_batch(n_ped)]
    temps = [0.3 ** (j / 7) for j in range(chains)]
    ctxs = []
    for pd in probs:
        ctx = api.Context(api.Problem.from_arrays(pd, with_legal=False), n_chains=chains, device=device,
                          lod_precision=api.SL_LOD_FP32_RESCALED, sampler_precision=api.SL_SAMPLER_FAST,
                          lod_flags=api.SL_LOD_ZERO_OK, lod_kernel=api.SL_LOD_KERNEL_INTERP)
        ctx.set_temperatures(temps)
        ctx.set_graphs(np.stack([pd["dg0"]] * chains))
        ctxs.append(ctx)
    setup_s = time.perf_counter() - t0
    opts = dict(burnin=0, period=10, lprob=LPROB, seed=SEED, exchange_period=10)
    with api.Batch(ctxs) as b:
        b.run(iterations=10, **opts)                      # builds the graph, warms up
        for c in ctxs:
            c.synchronize()
        t = time.perf_counter()
        b.run(iterations=10 + K, first_iteration=10, **opts)
        for c in ctxs:
            c.synchronize()
        dt = time.perf_counter() - t
    acc = sum(int(c.mc3_stats()[0].sum()) for c in ctxs)
    prop = sum(int(c.mc3_stats()[1].sum()) for c in ctxs)
    sizes = [pd["N"] for pd in probs]
    for c in ctxs:
        c.close()
    return {"value": K * chains * n_ped / dt, "unit": "chain-steps/s", "pedigrees": n_ped, "chains_per_pedigree": chains,
            "members": [min(sizes), max(sizes)], "markers": 1000, "iterations_timed": K,
            "exchanges_accepted": acc, "exchanges_proposed": prop, "setup_s": round(setup_s, 1),
            "timing": "wall clock around sl_batch_run + synchronize (host-side MC3 exchanges included)"}


def adjoint_rate(d, graphs, device):
    from swiftlink_gb300 import api
    from swiftlink_gb300.workloads import disease_probs
    pen, q = (0.01, 0.8, 0.9), 1e-3
    dd = dict(d, penetrance=np.array(pen), freq=np.float64(q),
              disease_prob=disease_probs(d["affection"], d["mother"] < 0, q, pen))
    npos = (d["M"] - 1) * d["n_lod"]
    with api.Context(api.Problem.from_arrays(dd, with_legal=False), n_chains=1, device=device,
                     lod_precision=api.SL_LOD_FP32_RESCALED, lod_flags=api.SL_LOD_ZERO_OK) as ctx:
        ctx.trait_backward(graphs[:1])
        reps = 3
        t = time.perf_counter()
        for _ in range(reps):
            grad, pt = ctx.trait_backward(graphs)
        dt = (time.perf_counter() - t) / reps
    return {"value": graphs.shape[0] * npos / dt, "unit": "positions/s", "graphs": int(graphs.shape[0]),
            "model": "dominant (0.01, 0.8, 0.9), q = 1e-3",
            "path": "sl_trait_backward: host graphs in, d log L / d (theta_L, theta_R, penetrances, q) out"}


def timed_lod(ctx, stream, flush, G, npos, reps):
    import torch
    ctx.lod_score_chains()
    ctx.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for i in range(reps):
        with torch.cuda.stream(stream):
            flush.fill_(i)
            evs[i][0].record(stream)
        ctx.lod_score_chains()
        with torch.cuda.stream(stream):
            evs[i][1].record(stream)
    ctx.synchronize()
    t = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    return reps * G * npos / t


def inst_from_profiles(name):
    """Warp instructions per launch (smsp__inst_executed.sum) from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("| smsp__inst_executed.sum |"):
            try:
                return float(line.split("|")[2].split()[0].replace(",", ""))
            except (ValueError, IndexError):
                return None
    return None


def issue_estimate(C, it0, it1, seed, lprob, n_meioses, sm_mhz, sms, seconds):
    """SM issue utilisation of timed run-graph launches on the 120-member,
    2,000-SNP workload: the warp instructions of the L- and M-sweeps they ran
    (each chain's L/M choice replayed with the same Philox draws; instructions
    per sweep from the committed ncu summaries of this workload's kernels) over
    the SMs' issue rate (4 schedulers per SM, one warp instruction per cycle
    each, at the SM clock sampled during the launches)."""
    from swiftlink_gb300 import philox
    ls = inst_from_profiles("sl_ls_jit_cfg2.md")           # one half-sweep (1,000 loci) of 10 chains
    fag = inst_from_profiles("fag_warp_kernel_cfg2.md")    # one meiosis step of one chain
    scan = inst_from_profiles("ffbs_scan_kernel_cfg2.md")  # one meiosis step of one chain
    if None in (ls, fag, scan) or not sm_mhz or not sms or seconds <= 0:
        return None
    c = np.arange(C, dtype=np.uint64)[:, None]
    it = np.arange(it0, it1, dtype=np.uint64)[None, :]
    hi = (c << np.uint64(40)) ^ (it << np.uint64(4)) ^ np.uint64(7)
    n_l = int((philox.uniform(seed, hi, 0) < lprob).sum())
    n_m = C * (it1 - it0) - n_l
    per_l = 2 * ls / 10                                  # both halves, one chain
    per_m = (n_meioses + 1) * fag + n_meioses * scan     # a reset launch, then a likelihood and a scan per meiosis
    inst = n_l * per_l + n_m * per_m
    peak = sms * 4 * sm_mhz * 1e6
    return {"bound": "issue", "achieved": inst / seconds / 1e9, "peak": peak / 1e9, "unit": "G warp-inst/s",
            "frac": inst / seconds / peak, "l_sweeps": n_l, "m_sweeps": n_m,
            "warp_inst_per_l_sweep": per_l, "warp_inst_per_m_sweep": per_m,
            "source": "instructions per launch: smsp__inst_executed.sum in profiles/sl_ls_jit_cfg2.md, "
                      "fag_warp_kernel_cfg2.md, ffbs_scan_kernel_cfg2.md; the scoring launches are left out"}


def traffic_from_profiles(kernel):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    path = os.path.join(ROOT, "profiles", "traffic.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("|") and kernel in line:
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            try:
                return float(cells[-1])
            except ValueError:
                return None
    return None


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
