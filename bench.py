#!/usr/bin/env python
"""Benchmark of the SwiftLink MCMC hot path on GB300.

Workload (headline): the seeded synthetic 400-member, 8-generation pedigree
with 10 consanguinity loops and 60 affected, 10,000 SNPs at 0.1 cM, recessive
model, 32 replicate chains per GPU, scoring every 100th descent graph at 5
positions per marker interval (49,995 LOD positions per scored graph): the
largest workload that fits one GPU.

A step is 5 MCMC iterations (MarkovChain::run, markov_chain.cc:335-392) of
every chain -- each an L-sweep over all 10,000 loci or an M-sweep over all
non-ignorable meioses, chosen per chain with probability 0.5 -- plus LOD
scoring on iterations that are multiples of 100; the timed window starts at
iteration 100, so the 20 default steps score every chain once.  `value` is
descent-graph steps/s (chain-iterations/s) over all chains and GPUs, batched
form (all chains in one launch of the run graph, FP32 samplers, FP32-rescaled
LOD peel with FP64 log-sums).  LOD positions/s, the plain single-chain form,
the 120-member workload, the trait-peel adjoint on 1,000 graphs and the
uneven 64-pedigree MC3 batch are reported beside it.

Arms:
  python bench.py [--gpus N --steps K --warmup W]   this implementation
  python bench.py --impl reference ...               the reference's CPU path
      on the host cores: the C restatement in oracle/ (the reference's own
      program does not build on the Arm host), one process per core, each
      timing bounded slices of the same workload's sweeps and scoring
"""
from __future__ import annotations

import argparse
import json
import math
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
CHAINS = 32
PERIOD = 100
STEP_ITERS = 5        # MCMC iterations of every chain per timed step
LPROB = 0.5
SEED = 20261205
L2_FLUSH_BYTES = 256 << 20  # larger than the 129 MB L2
# bounded slices of the CPU arms
SLICE_LOCI = 100
SLICE_MEIOSES = 4
SLICE_INTERVALS = 100
REF_BUDGET_S = 150.0
DLOD_INTERVALS = (4000, 4040)   # the oracle's check of the FP32 table: 200 positions


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--skip-extras", action="store_true",
                    help="leave out the 120-member, adjoint and uneven-batch measurements")
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


def window(W, K):
    """First iteration of the timed window (a multiple of the scoring period,
    so the window scores every chain) and of the warm-up before it."""
    it0 = PERIOD * max(1, math.ceil(W * STEP_ITERS / PERIOD))
    return it0, it0 - W * STEP_ITERS


def config(world):
    return {"workload": "400-member 8-generation pedigree, 10 loops, 60 affected, 10000 SNPs at 0.1 cM, "
                        "recessive (0,0,1) q=1e-4, 32 replicate chains per GPU, scoring every 100th graph, "
                        "5 LOD positions per interval",
            "members": 400, "markers": 10000, "chains_per_gpu": CHAINS, "scoring_period": PERIOD,
            "lod_positions_per_graph": 49995, "lsampler_prob": LPROB,
            "parallelism": f"replicas x{world}",
            "step": f"{STEP_ITERS} MCMC iterations of every chain in one run-graph launch; the window starts at "
                    f"iteration {PERIOD}, so it scores every chain's graph once; value = chain-iterations/s",
            "l2": "flushed (256 MB write) before every timed step",
            "zero_likelihood_positions": "counted as zero terms of the log-sum (SL_LOD_ZERO_OK); the FP32-"
                                         "rescaled peel finds none on this pedigree"}


def headline_problem():
    from swiftlink_gb300 import pedigree, synth
    return pedigree.problem_from_workload(synth.make_workload(5))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.ids = [str(device)]
        try:   # the GPU this process runs on, whatever CUDA_VISIBLE_DEVICES maps
            import torch
            u = str(torch.cuda.get_device_properties(device).uuid)
            self.ids.insert(0, u if u.startswith("GPU-") else "GPU-" + u)
        except Exception:
            pass
        self.proc = None
        self.path = None

    def start(self):
        for gid in self.ids:
            try:
                fd, self.path = tempfile.mkstemp(suffix=".csv")
                os.close(fd)
                self.f = open(self.path, "w")
                self.proc = subprocess.Popen(["nvidia-smi", f"--id={gid}", f"--query-gpu={self.QUERY}",
                                              "--format=csv,noheader,nounits", "-lms", "200"],
                                             stdout=self.f, stderr=subprocess.DEVNULL)
                time.sleep(0.3)
                if self.proc.poll() is None:
                    return
                self.f.close()
                os.unlink(self.path)
            except Exception:
                pass
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
# CPU arms: the C restatement of the reference (oracle/), bounded slices
# ---------------------------------------------------------------------------
def legal_masks(d):
    """Genotype elimination's masks of the problem (the library's host-side
    elimination, equal to the reference's GenotypeElimination): input tables
    of the CPU port, computed before any timing."""
    import ctypes
    from swiftlink_gb300 import api
    desc = api.Problem.from_arrays(d, with_legal=False).desc()
    out = np.zeros((d["M"], d["N"]), np.uint8)
    rc = api.lib().sl_problem_legal_masks(ctypes.byref(desc), out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError(f"sl_problem_legal_masks failed ({rc})")
    return out


def cpu_problem(d=None):
    from oracle import port
    d = dict(headline_problem() if d is None else d)
    d["legal"] = legal_masks(d)
    d["trait_prior"] = port.derive_priors(d["genotypes"], d["typed"], d["minor"])
    return d


def slice_times(P, d, dg, chain, rounds, budget_s, seed=SEED):
    """Time bounded slices of one chain's work on the CPU port, with the
    device driver's Philox draws: L-steps at SLICE_LOCI consecutive even loci
    (slo_lsteps, in place), an M-sweep over SLICE_MEIOSES meioses of the
    shuffled order (slo_msweep), and the rescaled FP64 trait peel of
    SLICE_INTERVALS intervals.  Returns seconds per full L-sweep, per full
    M-sweep and per scoring of one graph, extrapolated by the slices' share."""
    from swiftlink_gb300 import philox
    M, K, N = d["M"], d["K"], d["N"]
    nm = len(d["meioses"])
    tl = tm = ts = 0.0
    nl = nmm = ns = 0
    t_start = time.perf_counter()
    for r in range(rounds):
        it = PERIOD + r
        lo = (2 * SLICE_LOCI * r) % (M - 2 * SLICE_LOCI)
        loci = np.arange(lo, lo + 2 * SLICE_LOCI, 2, dtype=np.int32)
        u = philox.uniform(seed, philox.stage_hi(chain, it, 1),
                           (loci.astype(np.uint64)[:, None] << np.uint64(24))
                           ^ np.arange(K + 2 * N, dtype=np.uint64)[None, :])
        t = time.perf_counter()
        P.lsteps(dg, loci, u)
        tl += time.perf_counter() - t
        nl += loci.size
        order = philox.shuffled(seed, chain, it, d["meioses"])[:SLICE_MEIOSES]
        um = philox.msweep_draws(seed, chain, it, order.size, M)
        t = time.perf_counter()
        dg2, _ = P.msweep(dg, order, um)
        tm += time.perf_counter() - t
        nmm += order.size
        dg[...] = dg2
        l0 = (SLICE_INTERVALS * r) % (M - 1 - SLICE_INTERVALS)
        t = time.perf_counter()
        P.lod_range(dg[None], l0, l0 + SLICE_INTERVALS, rescale=True, zero_ok=True)
        ts += time.perf_counter() - t
        ns += SLICE_INTERVALS
        if time.perf_counter() - t_start > budget_s:
            break
    return {"lsweep_s": tl / nl * M, "msweep_s": tm / nmm * nm, "score_s": ts / ns * (M - 1),
            "loci": nl, "meioses": nmm, "intervals": ns}


def per_iteration_s(t, lprob=LPROB):
    """CPU seconds of one chain-iteration: an L- or M-sweep by the run's
    choice probability, and the scoring of every PERIOD-th graph."""
    return lprob * t["lsweep_s"] + (1 - lprob) * t["msweep_s"] + t["score_s"] / PERIOD


def cpu_baseline_sample(d, graphs, table32):
    """About 10-30 s of single-core CPU work on the same workload: slices of
    L-steps, M-sweep steps and scoring timed on the port and extrapolated to
    chain-iterations/s; plus the oracle's check of the device's FP32 LOD table
    (one scoring of every chain's graph) on 200 positions."""
    from oracle import port
    port.build()
    dc = cpu_problem(d)
    P = port.Port(dc)
    dg = np.ascontiguousarray(graphs[0], np.int32).copy()
    t = slice_times(P, dc, dg, 0, rounds=10, budget_s=20.0)
    rate = 1.0 / per_iteration_s(t)
    l0, l1 = DLOD_INTERVALS
    raw, cnt, tp = P.lod_range(graphs, l0, l1, rescale=True)
    from swiftlink_gb300 import api
    want = api.lod_table(raw, cnt, tp)
    n = d["n_lod"]
    dlod = float(np.abs(table32[l0 * n:l1 * n] - want).max())
    return {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
            "lod_positions_per_s": 1.0 / (t["score_s"] / ((d["M"] - 1) * n)),
            "sample": f"one chain, single thread: L-steps at {t['loci']} loci, M-sweep steps of {t['meioses']} "
                      f"meioses over all loci, rescaled FP64 scoring of {t['intervals']} intervals; extrapolated "
                      f"to {t['lsweep_s']:.1f} s per L-sweep, {t['msweep_s']:.1f} s per M-sweep, "
                      f"{t['score_s']:.1f} s per scoring",
            "max_abs_dlod_vs_oracle": dlod,
            "dlod_check": f"device FP32-rescaled table of one scoring of all {graphs.shape[0]} chains' graphs "
                          f"against the oracle's rescaled FP64 peel of the same graphs, intervals [{l0}, {l1})"}


def _ref_worker(args):
    chain, rounds, budget_s = args
    from oracle import port
    d = cpu_problem()
    P = port.Port(d)
    dg = np.ascontiguousarray(d["dg0"], np.int32).copy()
    t0 = time.perf_counter()
    t = slice_times(P, d, dg, chain, rounds, budget_s)
    t["wall"] = time.perf_counter() - t0
    return t


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import port
    port.build()
    cores = os.cpu_count() or 1
    workers = max(1, min(cores, CHAINS * args.gpus))
    rounds = max(1, args.steps + args.warmup)
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(workers) as pool:
        res = pool.map(_ref_worker, [(w, rounds, REF_BUDGET_S) for w in range(workers)])
    wall = time.perf_counter() - t0
    it_s = float(np.mean([per_iteration_s(t) for t in res]))   # CPU seconds per chain-iteration
    value = workers / it_s
    step_s = CHAINS * args.gpus * STEP_ITERS * it_s / workers
    lsw = float(np.mean([t["lsweep_s"] for t in res]))
    msw = float(np.mean([t["msweep_s"] for t in res]))
    sc = float(np.mean([t["score_s"] for t in res]))
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * step_s,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64 (samplers, peel and log-sums)",
           "data": "synthetic (seeded generator, swiftlink_gb300/synth.py)", "config": config(args.gpus),
           "lod_positions_per_s": workers * 49995 / sc,
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                            "sample": f"C restatement of the reference, {workers} processes (one chain each), "
                                      f"slices per process: L-steps at {res[0]['loci']} loci, M-sweep steps of "
                                      f"{res[0]['meioses']} meioses over all 10000 loci, rescaled FP64 scoring of "
                                      f"{res[0]['intervals']} intervals (capped at {REF_BUDGET_S:.0f} s); per chain "
                                      f"{lsw:.2f} s per L-sweep, {msw:.2f} s per M-sweep, {sc:.2f} s per scoring; "
                                      f"wall {wall:.1f} s"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# this implementation
# ---------------------------------------------------------------------------
def counters():
    """ncu figures of the kernels (DRAM bytes and warp instructions per
    launch, with the workload each was captured on), if recorded."""
    path = os.path.join(ROOT, "profiles", "counters.json")
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def lm_choices(C, it0, it1, seed, lprob):
    """Per iteration of [it0, it1), how many chains chose the L-sampler
    (the run's Philox choice replayed)."""
    from swiftlink_gb300 import philox
    c = np.arange(C, dtype=np.uint64)[:, None]
    it = np.arange(it0, it1, dtype=np.uint64)[None, :]
    hi = (c << np.uint64(40)) ^ (it << np.uint64(4)) ^ np.uint64(7)
    return (philox.uniform(seed, hi, 0) < lprob).sum(axis=0)


def issue_estimate(C, it0, it1, seed, lprob, n_meioses, sm_mhz, sms, seconds, counts, lanes=None, shares=None):
    """SM issue utilisation of timed run-graph launches: the warp instructions
    of the L- and M-sweeps they ran (each chain's L/M choice replayed with the
    same Philox draws; instructions per unit from ncu counts of the same
    workload: one chain's L half-sweep with the lane group in use, one chain's
    meiosis step in the founder-allele-graph and filter kernels) over the SMs'
    issue rate (4 schedulers per SM, one warp instruction per cycle each, at
    the SM clock sampled during the launches).  The scoring launches are left
    out.  With `shares` (each class's share of a profiled pass's kernel time)
    each class's instructions are also set against its share of the time."""
    need = ("fag_per_meiosis_step", "scan_per_meiosis_step")
    if not counts or any(counts.get(k) is None for k in need) or not sm_mhz or not sms or seconds <= 0:
        return None
    per_half = counts.get("l_half_sweep_per_chain")
    if per_half is None:
        per_half = (counts.get("l_half_sweep_per_chain_by_lanes") or {}).get(str(lanes))
    if per_half is None:
        return None
    n_l = int(lm_choices(C, it0, it1, seed, lprob).sum())
    n_m = C * (it1 - it0) - n_l
    per_l = 2 * per_half
    per_m = (n_meioses + 1) * counts["fag_per_meiosis_step"] + n_meioses * counts["scan_per_meiosis_step"]
    inst = n_l * per_l + n_m * per_m
    peak = sms * 4 * sm_mhz * 1e6
    out = {"bound": "issue", "achieved": inst / seconds / 1e9, "peak": peak / 1e9, "unit": "G warp-inst/s",
           "frac": inst / seconds / peak, "l_sweeps": n_l, "m_sweeps": n_m, "lsampler_lanes": lanes,
           "warp_inst_per_l_sweep": per_l, "warp_inst_per_m_sweep": per_m,
           "source": counts.get("source", "ncu smsp__inst_executed.sum")}
    if shares and shares.get("l") and shares.get("m"):
        out["frac_l_sweeps"] = n_l * per_l / (shares["l"] * seconds * peak)
        out["frac_m_sweeps"] = n_m * per_m / (shares["m"] * seconds * peak)
        out["class_fractions"] = "each class's instructions over its share of a profiled pass's kernel time " \
                                 "(the classes overlap in the timed run: approximate)"
    return out


def timed_lod(ctx, stream, flush, G, npos, reps, allmax=None):
    """Positions/s of one scoring of the context's chains (reps timed
    scorings, L2 flushed before each), the time the slowest rank's when
    allmax reduces over ranks."""
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
    if allmax is not None:
        t = allmax(t)
    return reps * G * npos / t


def run_ours(args):
    import torch
    from swiftlink_gb300 import api
    from swiftlink_gb300.workloads import step_bytes, position_bytes

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

    t_setup = time.perf_counter()
    d = headline_problem()
    setup_s = time.perf_counter() - t_setup
    prob = api.Problem.from_arrays(d, with_legal=False)
    N, F, M, n = d["N"], d["F"], d["M"], d["n_lod"]
    nm = len(d["meioses"])
    npos = (M - 1) * n
    C = CHAINS
    S = STEP_ITERS
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    seed = SEED + 7919 * rank
    W, K = args.warmup, args.steps
    it0, itw = window(W, K)
    run = dict(burnin=0, period=PERIOD, lprob=LPROB, seed=seed)

    # ---------------- batched form: all chains per launch, FP32 samplers, FP32-rescaled LOD
    ctx = api.Context(prob, n_chains=C, lod_precision=api.SL_LOD_FP32_RESCALED, device=local,
                      sampler_precision=api.SL_SAMPLER_FAST, lod_flags=api.SL_LOD_ZERO_OK,
                      ls_kernel=api.SL_LS_KERNEL_GENERIC)
    ctx.set_graphs(np.stack([d["dg0"]] * C))
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    ctx.run(iterations=it0, first_iteration=itw, **run)
    ctx.synchronize()
    ctx.lod_reset()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = Clocks(local)
    launches0 = ctx.launches
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    for i in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xff)
            ev[i][0].record(stream)
        ctx.run(iterations=it0 + (i + 1) * S, first_iteration=it0 + i * S, **run)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    gpu_launches = ctx.launches - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_s = allmax(sum(step_ms) / 1e3)
    value = K * S * C * world / t_s
    raw_run, cnt_run, tp_run = ctx.lod_results()
    graphs = ctx.get_graphs()

    # ---------------- kernel shares and the dominant kernel's roofline, from a profiled
    # pass: the same kind of iterations, kernels launched one by one with per-class events
    itp = it0 + K * S
    Kp = 2
    ctx.profile(True)
    ctx.run(iterations=itp + Kp, first_iteration=itp, **dict(run, period=1 << 30))
    ctx.synchronize()
    kern = {k: ctx.profile_read(k) for k in range(5)}
    ctx.profile(False)
    n_l = lm_choices(C, itp, itp + Kp, seed, LPROB)
    per_locus = -(-N // 4) + 2 * (-(-(N - F) // 4)) + 8
    sb = step_bytes(N, F, M)
    classes = {
        0: ("lsampler_kernel<float> (one half-sweep of the chains that chose L)",
            float(n_l.sum()) * (M // 2) * per_locus / max(1, kern[0][1])),
        1: ("M-sweep graph (fag_warp_kernel + ffbs_scan_kernel, every meiosis of the chains that chose M)",
            float((C - n_l).sum()) * sb / max(1, kern[1][1])),
    }
    tot = max(1e-9, sum(x[0] for x in kern.values()))
    names = {0: "lsampler_kernel", 1: "fag_warp_kernel+ffbs_scan_kernel", 2: "LOD scoring kernel",
             3: "lod_merge_kernel", 4: "choose/shuffle"}
    dom = 0 if kern[0][0] >= kern[1][0] else 1
    dom_name, dom_bytes = classes[dom]
    dom_s = kern[dom][0] / 1e3 / max(1, kern[dom][1])
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(peaks_path)) if os.path.exists(peaks_path) else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = dom_bytes / dom_s / 1e9
    cnt = counters()
    ck = cnt.get("lsampler_kernel_cfg5" if dom == 0 else "msweep_cfg5", {})
    traffic = None
    if ck.get("dram_bytes_per_unit") is not None:
        units = float(n_l.sum()) * (M // 2) / max(1, kern[0][1]) if dom == 0 else \
            float((C - n_l).sum()) / max(1, kern[1][1])
        traffic = ck["dram_bytes_per_unit"] * units
    roofline = {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks
                else "of fallback (6.8 TB/s)",
                "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": 1e3 * dom_s,
                "bytes_per_unit": per_locus if dom == 0 else sb,
                "unit_of_work": "one (chain, locus) L-step: 2-bit genotypes of every member, the non-founder "
                                "indicators read and written, 8 bytes of map" if dom == 0 else
                                "one chain's M-sweep: every locus's genotypes, indicators read and written, map",
                "traffic_source": ck.get("source"),
                "note": "latency- and issue-bound integer and FP32 work on small rfunctions: the HBM fraction is "
                        "small by construction; the issue estimate below is the binding bound",
                "kernel_share_profiled_pass": {names[k]: round(v[0] / tot, 4) for k, v in kern.items()}}
    try:
        ktot = max(1e-9, kern[0][0] + kern[1][0])
        roofline["issue"] = issue_estimate(C, it0, it0 + K * S, seed, LPROB, nm, (clk or {}).get("sm_mhz"),
                                           torch.cuda.get_device_properties(dev).multi_processor_count,
                                           sum(step_ms) / 1e3, cnt.get("issue_cfg5"), ctx.ls_tuning()[0],
                                           {"l": kern[0][0] / ktot, "m": kern[1][0] / ktot})
    except Exception as exc:   # an estimate only: never lose the bench line over it
        roofline["issue"] = {"error": str(exc)[:200]}

    # ---------------- LOD positions/s: batched (all chains' graphs per launch, FP32-rescaled)
    # against plain (one graph per launch, FP64 with rescaling: the plain FP64 peel
    # underflows at every position of this pedigree, as the reference's does)
    lod_pos_s = timed_lod(ctx, stream, flush, C, npos, reps=5, allmax=allmax)
    lsel, ljit_ms = ctx.lod_kernel_info()
    ls_lanes, ls_t = ctx.ls_tuning()
    pctx = api.Context(prob, n_chains=1, lod_precision=api.SL_LOD_FP64_RESCALED, device=local,
                       lod_flags=api.SL_LOD_ZERO_OK)
    pctx.set_graphs(graphs[:1])
    pstream = torch.cuda.ExternalStream(pctx.stream_handle())
    plain_lod_pos_s = timed_lod(pctx, pstream, flush, 1, npos, reps=3, allmax=allmax)

    # ---------------- FP32 error: one scoring of the chains' graphs in FP32 against FP64 with rescaling
    ctx.lod_reset()
    ctx.lod_score_graphs(graphs)
    raw32, c32, tp32 = ctx.lod_results()
    table32 = api.lod_table(raw32, c32, tp32)
    with api.Context(prob, n_chains=C, lod_precision=api.SL_LOD_FP64_RESCALED, device=local,
                     lod_flags=api.SL_LOD_ZERO_OK) as p64:
        p64.set_graphs(graphs)
        p64.lod_score_chains()
        raw64, c64, tp64 = p64.lod_results()
    fin = raw64 > -1e300
    dlod = float(np.abs(table32 - api.lod_table(raw64, c64, tp64))[fin].max())
    with api.Context(prob, n_chains=1, lod_precision=api.SL_LOD_FP64, device=local,
                     lod_flags=api.SL_LOD_ZERO_OK) as plain64:
        plain64.set_graphs(graphs[:1])
        plain64.lod_score_chains()
        rawp, _, _ = plain64.lod_results()
    plain_underflow = int((rawp <= -1e300).sum())

    # ---------------- plain form: one chain, exact FP64 samplers, FP64-rescaled LOD
    xctx = api.Context(prob, n_chains=1, lod_precision=api.SL_LOD_FP64_RESCALED, device=local,
                       lod_flags=api.SL_LOD_ZERO_OK)
    xctx.set_graphs(graphs[:1])
    xstream = torch.cuda.ExternalStream(xctx.stream_handle())
    xctx.run(iterations=it0, first_iteration=it0 - 1, **run)
    xctx.synchronize()
    Kx = 3
    evx = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(Kx)]
    for i in range(Kx):
        with torch.cuda.stream(xstream):
            flush.fill_(i & 0xff)
            evx[i][0].record(xstream)
        xctx.run(iterations=it0 + i + 1, first_iteration=it0 + i, **run)
        with torch.cuda.stream(xstream):
            evx[i][1].record(xstream)
    xctx.synchronize()
    plain_steps_s = Kx / allmax(sum(a.elapsed_time(b) for a, b in evx) / 1e3)
    xctx.close()

    # ---------------- end to end through the public API with host buffers: every step
    # uploads the chains' graphs (H2D), runs the step's iterations and reads them back (D2H)
    host_graphs = graphs.copy()
    Ke = min(K, 6)
    ite = it0 + K * S + Kp
    barrier()
    t0 = time.perf_counter()
    for i in range(Ke):
        ctx.set_graphs(host_graphs)
        ctx.run(iterations=ite + (i + 1) * S, first_iteration=ite + i * S, **run)
        ctx.get_graphs(out=host_graphs)
    e2e_t = allmax(time.perf_counter() - t0)
    words = M * ((2 * (N - F) + 31) // 32)
    e2e = {"value": Ke * S * C * world / e2e_t, "unit": UNIT, "h2d_bytes_per_step": 4 * words * C,
           "d2h_bytes_per_step": 4 * words * C,
           "path": f"sl_set_descent_graphs (packed on the host, pinned copy) + sl_run ({S} iterations of "
                   f"{C} chains) + sl_get_descent_graphs per step, wall clock"}

    extras = {}
    if not args.skip_extras:
        extras["cfg2"] = cfg2_rate(local, dist, dev)
        extras["adjoint_cfg4"] = adjoint_rate(local)
        extras["uneven_batch_cfg3"] = uneven_batch_rate(local, dist, dev)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": t_s * 1e3 / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32 samplers (L-sampler, founder-allele graphs, meiosis filter) and f32 trait peel "
                        "with power-of-two rescaling; f64 LOD log-sums",
               "data": "synthetic (seeded generator, swiftlink_gb300/synth.py; no public dataset)",
               "config": config(world), "impl": "ours",
               "setup_s": round(setup_s, 1),
               "timed_window": {"iterations": [it0, it0 + K * S], "scored_graphs": int(cnt_run),
                                "steps_ms": [round(x, 2) for x in step_ms]},
               "lod_positions_per_s": lod_pos_s * world,
               "lod_kernel": {"selected": int(lsel), "specialised_compile_ms": round(ljit_ms, 1),
                              "selection": "timed at the first scoring (SL_LOD_KERNEL_AUTO)"},
               "ls_kernel": {"selected": "lsampler_kernel<float> (compact rfunctions)", "lanes": ls_lanes,
                             "timed_half_sweep_ms": {"32": round(ls_t[0], 3), "16": round(ls_t[1], 3),
                                                     "8": round(ls_t[2], 3)},
                             "selection": "SL_LS_KERNEL_GENERIC: 32, 16 or 8 lanes per (chain, locus) task, "
                                          "timed before the first sweep"},
               "plain": {"steps_per_s": plain_steps_s * world, "lod_positions_per_s": plain_lod_pos_s * world,
                         "form": "one chain per launch, exact FP64 samplers, FP64 LOD peel with rescaling",
                         "plain_fp64_positions_underflowed": plain_underflow},
               "batched_vs_plain": {"steps": value / (plain_steps_s * world),
                                    "lod_positions": lod_pos_s / plain_lod_pos_s},
               "max_abs_dlod_fp32_vs_fp64_rescaled": dlod,
               "gpu_launches": int(gpu_launches), "roofline": roofline, "clocks": clk, "e2e": e2e}
        out.update(extras)
        if world == 1:
            out["cpu_baseline"] = cpu_baseline_sample(d, graphs, table32)
        print(json.dumps(out))
    for c in (ctx, pctx):
        c.close()
    if dist:
        dist.destroy_process_group()


def cfg2_rate(device, dist, dev, C=10, K=10, S=20):
    """The 120-member, 6-generation, 3-loop pedigree with 2,000 SNPs at 0.2 cM,
    10 chains: chain-iterations/s of K run-graph launches of S iterations each
    (CUDA events, L2 flushed), the L-sampler chosen by SL_LS_KERNEL_AUTO."""
    import torch
    from swiftlink_gb300 import api
    from swiftlink_gb300.workloads import load_problem
    d = load_problem("cfg2")
    t = time.perf_counter()
    ctx = api.Context(api.Problem.from_arrays(d, with_legal=False), n_chains=C, device=device,
                      lod_precision=api.SL_LOD_FP32_RESCALED, sampler_precision=api.SL_SAMPLER_FAST,
                      lod_flags=api.SL_LOD_ZERO_OK, ls_kernel=api.SL_LS_KERNEL_AUTO)
    create_s = time.perf_counter() - t
    ctx.set_graphs(np.stack([d["dg0"]] * C))
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    run = dict(burnin=0, period=PERIOD, lprob=LPROB, seed=SEED)
    ctx.run(iterations=PERIOD, first_iteration=PERIOD - 3 * S, **run)
    ctx.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for i in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xff)
            ev[i][0].record(stream)
        ctx.run(iterations=PERIOD + (i + 1) * S, first_iteration=PERIOD + i * S, **run)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    ctx.synchronize()
    ts = rank_max(sum(a.elapsed_time(b) for a, b in ev) / 1e3, dist, dev)
    sel, ms = ctx.ls_kernel_info()
    ctx.close()
    return {"value": K * S * C / ts, "unit": "chain-steps/s per GPU", "chains": C, "iterations_timed": K * S,
            "ls_kernel": "specialised (sl_ls_jit)" if sel == api.SL_LS_KERNEL_SPECIALISED else "generic",
            "ls_compile_ms": round(ms, 1), "context_create_s": round(create_s, 1)}


def adjoint_rate(device, G=1000, chunk=250):
    """The trait-peel adjoint on the 120-member, 2,000-SNP pedigree under the
    dominant model (0.01, 0.8, 0.9), q = 1e-3: 1,000 stored graphs (10 chains'
    graphs after 5 MCMC iterations, repeated) x 9,995 positions through
    sl_trait_backward with host graphs in and host gradients out, in chunks
    of 250 graphs; wall clock."""
    from swiftlink_gb300 import api
    from swiftlink_gb300.workloads import disease_probs, load_problem
    d = load_problem("cfg2")
    pen, q = (0.01, 0.8, 0.9), 1e-3
    dd = dict(d, penetrance=np.array(pen), freq=np.float64(q),
              disease_prob=disease_probs(d["affection"], d["mother"] < 0, q, pen))
    prob = api.Problem.from_arrays(dd, with_legal=False)
    with api.Context(prob, n_chains=10, device=device, sampler_precision=api.SL_SAMPLER_FAST,
                     lod_precision=api.SL_LOD_FP32_RESCALED, lod_flags=api.SL_LOD_ZERO_OK) as sctx:
        sctx.set_graphs(np.stack([d["dg0"]] * 10))
        sctx.run(iterations=5, burnin=0, period=1 << 30, lprob=LPROB, seed=SEED)
        base = sctx.get_graphs()
    gset = np.stack([base[i % 10] for i in range(chunk)])
    npos = (d["M"] - 1) * d["n_lod"]
    with api.Context(prob, n_chains=1, device=device, lod_precision=api.SL_LOD_FP32_RESCALED,
                     lod_flags=api.SL_LOD_ZERO_OK) as ctx:
        segs, used = ctx.adjoint_memory()
        ctx.trait_backward(gset[:10])
        ctx.profile(True)   # event marks around the adjoint's launches: the device's share of the wall time
        t = time.perf_counter()
        done = 0
        while done < G:
            grad, pt = ctx.trait_backward(gset[:min(chunk, G - done)])
            done += min(chunk, G - done)
        dt = time.perf_counter() - t
        kern_ms, kern_n = ctx.profile_read(api.SL_KERNEL_LOD)
        ctx.profile(False)
        form, warp_ms, thread_ms, spec_ms = ctx.adjoint_info()
        shapes, variant, regs, compile_ms = ctx.adjoint_kernel_info()
        # the forward FP32 scorer on the same graphs, for the ratio
        ctx.lod_score_graphs(gset)
        ctx.synchronize()
        t = time.perf_counter()
        ctx.lod_score_graphs(gset)
        ctx.synchronize()
        fwd = chunk * npos / (time.perf_counter() - t)
    return {"value": G * npos / dt, "unit": "positions/s", "graphs": G, "positions_per_graph": npos,
            "kernel_positions_per_s": G * npos / (kern_ms / 1e3) if kern_ms > 0 else None,
            "kernel_launches": int(kern_n),
            "forward_fp32_positions_per_s": fwd, "adjoint_segments": segs, "shared_bytes_per_warp": used,
            "form": {api.SL_ADJOINT_WARP: "one warp per position, shared memory",
                     api.SL_ADJOINT_THREAD: "one thread per position, global arena",
                     api.SL_ADJOINT_SPECIALISED: "the peel's adjoint compiled for the pedigree, one thread per "
                                                 "position, global arena"}.get(form, str(form)),
            "form_timing_ms": {"warp": round(warp_ms, 3), "thread": round(thread_ms, 3),
                               "specialised": round(spec_ms, 3),
                               "tasks": 65536, "selection": "timed on the first call's first tasks"},
            "specialised": {"shapes": shapes, "registers": regs, "compile_ms": round(compile_ms, 1),
                            "variant": {0: "4 blocks per SM", 1: "8 blocks per SM"}.get(variant, str(variant))},
            "model": "dominant (0.01, 0.8, 0.9), q = 1e-3",
            "path": "sl_trait_backward: host graphs in, d log L / d (theta_L, theta_R, penetrances, q) out"}


def uneven_batch_rate(device, dist, dev, n_ped=64, chains=8, K=20):
    """Chain-steps/s of the uneven batch: 64 seeded pedigrees of 20-150
    members (0-4 loops, 1,000 SNPs at 0.5 cM), 8 MC3 chains each at
    temperatures 0.3^(j/7), fast samplers, FP32 LOD (the slot-program
    interpreter: no per-pedigree compilation), exchange and scoring every 10
    iterations: all pedigrees, spurts and exchanges in one graph launch."""
    import torch
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
        launches0 = sum(c.launches for c in ctxs)
        t = time.perf_counter()
        b.run(iterations=10 + K, first_iteration=10, **opts)
        for c in ctxs:
            c.synchronize()
        dt = rank_max(time.perf_counter() - t, dist, dev)
    acc = sum(int(c.mc3_stats()[0].sum()) for c in ctxs)
    prop = sum(int(c.mc3_stats()[1].sum()) for c in ctxs)
    sizes = [pd["N"] for pd in probs]
    for c in ctxs:
        c.close()
    return {"value": K * chains * n_ped / dt, "unit": "chain-steps/s", "pedigrees": n_ped,
            "chains_per_pedigree": chains, "members": [min(sizes), max(sizes)], "markers": 1000,
            "iterations_timed": K, "exchanges_accepted": acc, "exchanges_proposed": prop,
            "setup_s": round(setup_s, 1),
            "timing": "wall clock around one sl_batch_run (one graph launch: every pedigree's spurts and MC3 "
                      "exchanges on the device) + synchronize"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
