"""GPU parity: the CUDA kernels, called through the C ABI, against the
reference's golden vectors and against the C restatement of the reference on
seeded inputs.

Bars: descent-graph updates bit-exact (integer work); FP64 LOD within
|dLOD| <= 1e-10; FP32-rescaled LOD within |dLOD| <= 1e-3 (the target stated
for the batched form).
"""
import numpy as np
import pytest

from conftest import CASES, load_golden
from swiftlink_gb300 import philox as philox_np
from oracle import port
from swiftlink_gb300 import api

pytestmark = pytest.mark.gpu

FP64_LOD_TOL = 1e-10
FP32_LOD_TOL = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()
    port.build()


def make_ctx(g, n_chains=1, precision=api.SL_LOD_FP64):
    return api.Context(api.Problem.from_arrays(g), n_chains=n_chains, lod_precision=precision)


def stride_of(g):
    return g["K"] + 2 * g["N"]


@pytest.mark.parametrize("name", CASES)
def test_lsteps_bit_exact(name):
    g = load_golden(name)
    with make_ctx(g) as ctx:
        ctx.set_graphs(g["dg0"])
        for i, l in enumerate(g["lstep_loci"]):
            u = np.zeros((1, g["M"], stride_of(g)))
            u[0, l] = g["lstep_u"][i]
            ctx.lsampler_loci([int(l)], u)
            assert np.array_equal(ctx.get_graphs()[0], g["lstep_after"][i]), f"locus {l}"


@pytest.mark.parametrize("name", CASES)
def test_lsweep_bit_exact(name):
    g = load_golden(name)
    with make_ctx(g) as ctx:
        ctx.set_graphs(g["dg0"])
        ctx.lsampler_sweep(g["lsweep_u"][None])
        assert np.array_equal(ctx.get_graphs()[0], g["lsweep_after"])


@pytest.mark.parametrize("name", CASES)
def test_msweep_bit_exact(name):
    g = load_golden(name)
    with make_ctx(g) as ctx:
        ctx.set_graphs(g["lsweep_after"])
        ctx.msampler_sweep(g["msweep_order"], g["msweep_u"][None])
        assert np.array_equal(ctx.get_graphs()[0], g["msweep_after"])


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision,tol", [(api.SL_LOD_FP64, FP64_LOD_TOL),
                                           (api.SL_LOD_FP32_RESCALED, FP32_LOD_TOL)])
def test_lod_against_reference(name, precision, tol):
    g = load_golden(name)
    with make_ctx(g, precision=precision) as ctx:
        ctx.lod_score_graphs(g["lod_graphs"])
        raw, cnt, tp = ctx.lod_results()
    assert cnt == g["lod_count"]
    assert abs(tp - g["lod_trait_prob"]) <= 1e-12 * max(1.0, abs(tp))
    got = api.lod_table(raw, cnt, tp)
    want = api.lod_table(g["lod_raw"], g["lod_count"], g["lod_trait_prob"])
    err = np.abs(got - want).max()
    assert err <= tol, err


@pytest.mark.parametrize("name", CASES)
def test_lod_chains_equals_graphs(name):
    """Scoring resident chains gives the same table as scoring uploaded graphs."""
    g = load_golden(name)
    graphs = g["lod_graphs"]
    with make_ctx(g, n_chains=graphs.shape[0]) as ctx:
        ctx.set_graphs(graphs)
        ctx.lod_score_chains()
        a = ctx.lod_results()
        ctx.lod_reset()
        ctx.lod_score_graphs(graphs)
        b = ctx.lod_results()
    np.testing.assert_array_equal(a[0], b[0])
    assert a[1] == b[1] == graphs.shape[0]


def test_multichain_batch_matches_port():
    g = load_golden("cfg1")
    P = port.Port(g)
    C = 4
    rng = np.random.default_rng(7)
    st = stride_of(g)
    ul = rng.random((C, g["M"], st))
    order = g["msweep_order"]
    um = rng.random((C, order.size, g["M"]))
    with make_ctx(g, n_chains=C) as ctx:
        ctx.set_graphs(np.stack([g["dg0"]] * C))
        ctx.lsampler_sweep(ul, n_chains=C)
        ctx.msampler_sweep(order, um, n_chains=C)
        out = ctx.get_graphs()
    for c in range(C):
        dg = g["dg0"].copy()
        for l in list(range(0, g["M"], 2)) + list(range(1, g["M"], 2)):
            dg, _ = P.lstep(dg, l, ul[c, l])
        dg, _ = P.msweep(dg, order, um[c])
        assert np.array_equal(out[c], dg), f"chain {c}"


from swiftlink_gb300.workloads import load_problem  # noqa: E402


def test_cfg2_seeded_against_port():
    """120 members, 2000 markers: sweeps bit-exact and LOD within tolerance."""
    d = load_problem("cfg2")
    prob = api.Problem.from_arrays(d, with_legal=False)
    C = 2
    with api.Context(prob, n_chains=C) as ctx:
        d["legal"] = ctx.legal_masks()
        d["trait_prior"] = ctx.trait_priors()
        P = port.Port(d)
        rng = np.random.default_rng(2)
        st = d["K"] + 2 * d["N"]
        ul = rng.random((C, d["M"], st))
        order = d["meioses"].copy()
        rng.shuffle(order)
        order = order[:24]
        um = rng.random((C, order.size, d["M"]))
        ctx.set_graphs(np.stack([d["dg0"]] * C))
        ctx.lsampler_sweep(ul, n_chains=C)
        ctx.msampler_sweep(order, um, n_chains=C)
        out = ctx.get_graphs()
        ctx.lod_score_chains()
        raw64, cnt, tp = ctx.lod_results()
    want = []
    for c in range(C):
        dg = d["dg0"].copy()
        for l in list(range(0, d["M"], 2)) + list(range(1, d["M"], 2)):
            dg, _ = P.lstep(dg, l, ul[c, l])
        dg, _ = P.msweep(dg, order, um[c])
        assert np.array_equal(out[c], dg), f"chain {c}"
        want.append(dg)
    ref_raw, ref_cnt, ref_tp = P.lod(np.stack(want))
    assert cnt == ref_cnt
    lod_ref = api.lod_table(ref_raw, ref_cnt, ref_tp)
    assert np.abs(api.lod_table(raw64, cnt, tp) - lod_ref).max() <= FP64_LOD_TOL
    with api.Context(prob, n_chains=C, lod_precision=api.SL_LOD_FP32_RESCALED) as c32:
        c32.set_graphs(np.stack(want))
        c32.lod_score_chains()
        raw32, cnt32, tp32 = c32.lod_results()
    assert np.abs(api.lod_table(raw32, cnt32, tp32) - lod_ref).max() <= FP32_LOD_TOL


def replay_run(P, g, dgs, seed, iters, lprob, period, burnin):
    """Host replay of sl_run's schedule with the same Philox streams."""
    M, K, N = g["M"], g["K"], g["N"]
    st = K + 2 * N
    base = g["meioses"]
    scored = []
    for it in range(iters + burnin):
        for c in range(len(dgs)):
            if philox_np.chooses_l(seed, c, it, lprob):
                u = philox_np.lsweep_draws(seed, c, it, M, st)
                for l in list(range(0, M, 2)) + list(range(1, M, 2)):
                    dgs[c], _ = P.lstep(dgs[c], l, u[l])
            else:
                order = philox_np.shuffled(seed, c, it, base)
                u = philox_np.msweep_draws(seed, c, it, order.size, M)
                dgs[c], _ = P.msweep(dgs[c], order, u)
        if it >= burnin and it % period == 0:
            scored.extend(d.copy() for d in dgs)
    return dgs, scored


@pytest.mark.parametrize("name", ["loop", "cfg1"])
def test_device_run_matches_host_replay(name):
    g = load_golden(name)
    P = port.Port(g)
    C, seed, iters, burnin, period = 3, 99, 6, 1, 2
    with make_ctx(g, n_chains=C) as ctx:
        ctx.set_graphs(np.stack([g["dg0"]] * C))
        ctx.run(iterations=iters, burnin=burnin, period=period, lprob=0.5, seed=seed)
        ctx.synchronize()
        out = ctx.get_graphs()
        raw, cnt, tp = ctx.lod_results()
    dgs, scored = replay_run(P, g, [g["dg0"].copy() for _ in range(C)], seed, iters, 0.5, period, burnin)
    for c in range(C):
        assert np.array_equal(out[c], dgs[c]), f"chain {c}"
    ref_raw, ref_cnt, ref_tp = P.lod(np.stack(scored))
    assert cnt == ref_cnt
    assert np.abs(api.lod_table(raw, cnt, tp) - api.lod_table(ref_raw, ref_cnt, ref_tp)).max() <= FP64_LOD_TOL


def test_illegal_graph_reports_error_and_context_recovers():
    g = load_golden("cfg1")
    P = port.Port(g)
    dg = g["dg0"].copy()
    # flip meioses until some column becomes illegal (zero founder-allele-graph likelihood)
    bad = None
    for l in range(g["M"]):
        for i in range(g["F"], g["N"]):
            for par in (0, 1):
                dg[l, i, par] ^= 1
                if P.fag(dg, l) == 0.0:
                    bad = (l, i, par)
                    break
                dg[l, i, par] ^= 1
            if bad:
                break
        if bad:
            break
    if bad is None:
        pytest.skip("no single flip makes this pedigree illegal")
    with make_ctx(g) as ctx:
        ctx.set_graphs(dg)
        order = g["msweep_order"]
        with pytest.raises(api.SwiftLinkError) as e:
            ctx.msampler_sweep(order, np.full((1, order.size, g["M"]), 0.5))
        assert e.value.code == api.SL_EILLEGAL
        ctx.set_graphs(g["lsweep_after"])
        ctx.msampler_sweep(order, g["msweep_u"][None])
        assert np.array_equal(ctx.get_graphs()[0], g["msweep_after"])


def test_rejects_interfering_loci():
    g = load_golden("loop")
    with make_ctx(g) as ctx:
        with pytest.raises(api.SwiftLinkError) as e:
            ctx.lsampler_loci([0, 1], np.zeros((1, g["M"], stride_of(g))))
        assert e.value.code == api.SL_EINVAL


# The fast (FP32) samplers round differently from the reference's FP64
# arithmetic, so a draw that falls within rounding distance of a decision
# boundary may go the other way.  The stated bound: a fast decision may differ
# from the exact one only where the exact draw lies within DECISION_MARGIN of
# its boundary (the FP32 sampling probabilities are within about 1e-6 of the
# FP64 ones; the M-sampler's scan compounds that along the map).
DECISION_MARGIN = 1e-4


def _seeded(name):
    if name == "cfg1":
        g = load_golden("cfg1")
        return g, g["lsweep_after"]
    if name == "cfg5":
        from swiftlink_gb300 import pedigree, synth
        g = pedigree.problem_from_workload(synth.make_workload(5))
        return g, g["dg0"]
    from swiftlink_gb300.workloads import load_problem
    g = load_problem("cfg2")
    return g, g["dg0"]


@pytest.mark.parametrize("name", ["cfg1", "cfg2"])
def test_fast_lsampler_decisions_match_exact(name):
    """Decision level, L-sampler (sampler_rfunction.cc:159-188,
    locus_sampler2.cc:44-65): over 10 sweeps, every half-sweep is run from the
    same graph in both modes with the same uniforms; each locus's new column
    (its meiosis indicators) must be equal in the two modes, or the exact
    step must have met a draw within DECISION_MARGIN of a cumulative boundary
    (the smallest such distance of the step, from the C restatement)."""
    g, state = _seeded(name)
    M, st = g["M"], stride_of(g)
    rng = np.random.default_rng(71)
    steps = differ = 0
    prob = api.Problem.from_arrays(g, with_legal=False)
    with api.Context(prob, n_chains=1) as ex, \
            api.Context(prob, n_chains=1, sampler_precision=api.SL_SAMPLER_FAST) as fa:
        g = dict(g, legal=ex.legal_masks(), trait_prior=ex.trait_priors())
        P = port.Port(g)
        state = np.ascontiguousarray(state, np.int32)
        for sweep in range(10):
            for parity in (0, 1):
                loci = np.arange(parity, M, 2, dtype=np.int32)
                u = rng.random((1, M, st))
                out = {}
                for mode, ctx in (("exact", ex), ("fast", fa)):
                    ctx.set_graphs(state[None])
                    ctx.lsampler_loci(loci, u)
                    out[mode] = ctx.get_graphs()[0]
                bad = [int(l) for l in loci if not np.array_equal(out["exact"][l], out["fast"][l])]
                for l in bad:
                    port.margin_reset()
                    P.lstep(state, l, u[0, l])
                    m = port.margin()
                    assert m < DECISION_MARGIN, f"sweep {sweep} locus {l}: columns differ, smallest margin {m:.3g}"
                steps += loci.size
                differ += len(bad)
                state = out["exact"]
    print(f"{name}: {differ} of {steps} fast L-steps differ from exact, each at a near-tie")
    assert differ <= steps // 100


@pytest.mark.parametrize("name", ["cfg1", "cfg2", "cfg5"])
def test_fast_msampler_decisions_match_exact(name):
    """Decision level, M-sampler (meiosis_sampler.cc:157-203): 40 meiosis
    steps (reset and step at one meiosis, the FP64 filter against the FP32
    founder-allele likelihoods and scan), each from the same graph with the
    same uniforms in both modes.  Backward sampling runs from the last locus
    down, so the first locus (from the top) where the two rows differ is
    where the decisions parted: the exact draw there must lie within
    DECISION_MARGIN of its threshold."""
    g, state = _seeded(name)
    M, F = g["M"], g["F"]
    rng = np.random.default_rng(72)
    prob = api.Problem.from_arrays(g, with_legal=False)
    differ = 0
    with api.Context(prob, n_chains=1) as ex, \
            api.Context(prob, n_chains=1, sampler_precision=api.SL_SAMPLER_FAST) as fa:
        g = dict(g, legal=ex.legal_masks(), trait_prior=ex.trait_priors())
        P = port.Port(g)
        state = np.ascontiguousarray(state, np.int32)
        meioses = rng.permutation(g["meioses"])[:12 if name == "cfg5" else 40]
        for m in meioses:
            u = rng.random((1, 1, M))
            out = {}
            for mode, ctx in (("exact", ex), ("fast", fa)):
                ctx.set_graphs(state[None])
                ctx.msampler_sweep([int(m)], u)
                out[mode] = ctx.get_graphs()[0]
            want, margins = port.msweep_margins(P, state, int(m), u[0, 0])
            assert np.array_equal(out["exact"], want)
            person, par = F + int(m) // 2, int(m) % 2
            rows = out["exact"][:, person, par], out["fast"][:, person, par]
            diff = np.nonzero(rows[0] != rows[1])[0]
            assert np.array_equal(np.delete(out["exact"], person, axis=1), np.delete(out["fast"], person, axis=1))
            if diff.size:
                top = int(diff.max())
                assert margins[top] < DECISION_MARGIN, f"meiosis {m}: rows part at locus {top}, margin {margins[top]:.3g}"
                differ += 1
            state = out["exact"]
    print(f"{name}: {differ} of {meioses.size} fast M-steps differ from exact, each from a near-tie")
    assert differ <= meioses.size // 4


@pytest.mark.parametrize("name", ["cfg1", "cfg2", "cfg5"])
@pytest.mark.parametrize("nchain", [1, 8])
def test_fast_msweep_equals_its_steps_one_by_one(name, nchain):
    """A fast M-sweep reuses, at each step, the likelihoods of the current
    column that the previous step computed (raw[l][current],
    meiosis_sampler.cc:123-124); a sweep of one meiosis computes them afresh.
    A sweep over 24 meioses must give the graph, bit for bit, that 24
    one-meiosis sweeps with the same uniforms give (8 chains: the
    founder-allele kernel's two-loci-per-warp form where a column fits)."""
    g, state = _seeded(name)
    M = g["M"]
    rng = np.random.default_rng(73)
    order = rng.permutation(g["meioses"])[:24].astype(np.int32)
    u = rng.random((nchain, order.size, M))
    prob = api.Problem.from_arrays(g, with_legal=False)
    with api.Context(prob, n_chains=nchain, sampler_precision=api.SL_SAMPLER_FAST) as fa:
        fa.set_graphs(np.stack([state] * nchain))
        fa.msampler_sweep(order, u, n_chains=nchain)
        whole = fa.get_graphs()
        fa.set_graphs(np.stack([state] * nchain))
        for j, m in enumerate(order):
            fa.msampler_sweep([int(m)], u[:, j:j + 1], n_chains=nchain)
        steps = fa.get_graphs()
    assert np.array_equal(whole, steps)
    assert not np.array_equal(whole[0], state)


def test_fast_and_exact_long_runs_agree_within_monte_carlo_error():
    """Long runs on the 30-member pedigree: 8 chains x 10 segments of 1,000
    iterations, scoring every 10th graph, in the exact mode (FP64 samplers and
    LOD) and in the fast mode (FP32 samplers, FP32-rescaled LOD), from the same
    seeds.  Each segment's LOD table is an estimate; the two modes' mean tables
    must agree within 5 combined standard errors at every position (the
    segments' spread gives the errors)."""
    g = load_golden("cfg1")
    C, segs, seg_it = 8, 10, 1000
    tables = {}
    for mode, kw in (("exact", {}), ("fast", dict(sampler_precision=api.SL_SAMPLER_FAST,
                                                  lod_precision=api.SL_LOD_FP32_RESCALED))):
        est = []
        with api.Context(api.Problem.from_arrays(g), n_chains=C, **kw) as ctx:
            ctx.set_graphs(np.stack([g["lsweep_after"]] * C))
            ctx.run(iterations=seg_it, burnin=0, period=10, lprob=0.5, seed=99)   # burn-in
            ctx.lod_reset()
            for s in range(segs):
                ctx.run(iterations=(s + 2) * seg_it, burnin=0, period=10, lprob=0.5, seed=99,
                        first_iteration=(s + 1) * seg_it)
                raw, cnt, tp = ctx.lod_results()
                assert cnt == C * seg_it // 10
                est.append(api.lod_table(raw, cnt, tp))
                ctx.lod_reset()
        tables[mode] = np.array(est)
    mean = {k: v.mean(0) for k, v in tables.items()}
    se = {k: v.std(0, ddof=1) / np.sqrt(segs) for k, v in tables.items()}
    comb = np.sqrt(se["exact"] ** 2 + se["fast"] ** 2)
    z = np.abs(mean["exact"] - mean["fast"]) / np.maximum(comb, 1e-6)
    print(f"max |mean dLOD| {np.abs(mean['exact'] - mean['fast']).max():.4f}, max z {z.max():.2f}, "
          f"median SE {np.median(comb):.4f}")
    assert z.max() <= 5.0


LOD_KERNELS = [api.SL_LOD_KERNEL_INTERP, api.SL_LOD_KERNEL_JIT_REG, api.SL_LOD_KERNEL_JIT_SMEM,
               api.SL_LOD_KERNEL_AUTO]


@pytest.mark.parametrize("kernel", LOD_KERNELS)
@pytest.mark.parametrize("name", CASES)
def test_batched_lod_kernels_against_reference(name, kernel):
    """Every kernel of the FP32-rescaled scorer (the slot-program interpreter,
    the problem-specialised forms with values in registers or in shared
    memory, and the timed choice) within |dLOD| <= 1e-3 of the reference."""
    g = load_golden(name)
    with api.Context(api.Problem.from_arrays(g), n_chains=1, lod_precision=api.SL_LOD_FP32_RESCALED,
                     lod_kernel=kernel) as ctx:
        ctx.lod_score_graphs(g["lod_graphs"][:1])
        ctx.lod_score_graphs(g["lod_graphs"][1:])
        raw, cnt, tp = ctx.lod_results()
        used, _ = ctx.lod_kernel_info()
    assert used != api.SL_LOD_KERNEL_AUTO
    if kernel != api.SL_LOD_KERNEL_AUTO:
        assert used == kernel
    assert cnt == g["lod_count"]
    got = api.lod_table(raw, cnt, tp)
    want = api.lod_table(g["lod_raw"], g["lod_count"], g["lod_trait_prob"])
    assert np.abs(got - want).max() <= FP32_LOD_TOL


_LARGE = {}


def large_pedigree_graphs():
    """The 120-member, 2000-SNP pedigree and four seeded graphs (the starting
    graph after 0-3 oracle L-sweeps) with the oracle's FP64 LOD of the set.
    Under the fully penetrant recessive model the second sweep's graph has
    positions of zero trait likelihood; the LOD counts them as zero terms."""
    if not _LARGE:
        from swiftlink_gb300.workloads import load_problem
        d = load_problem("cfg2")
        d["trait_prior"] = port.derive_priors(d["genotypes"], d["typed"], d["minor"])
        P = port.Port(d)
        rng = np.random.default_rng(31)
        st = d["K"] + 2 * d["N"]
        graphs = [d["dg0"].copy()]
        for _ in range(3):
            dg = graphs[-1].copy()
            u = rng.random((d["M"], st))
            for l in list(range(0, d["M"], 2)) + list(range(1, d["M"], 2)):
                dg, _ = P.lstep(dg, l, u[l])
            graphs.append(dg)
        graphs = np.stack(graphs)
        _LARGE.update(d=d, graphs=graphs, ref=P.lod(graphs, zero_ok=True))
    return _LARGE["d"], _LARGE["graphs"], _LARGE["ref"]


@pytest.mark.parametrize("kernel", LOD_KERNELS)
def test_batched_lod_kernels_large_pedigree(kernel):
    """Each batched kernel on the 120-member, 2000-SNP pedigree against the
    oracle's FP64 LOD, |dLOD| <= 1e-3, zero-likelihood positions counted as
    zero terms (SL_LOD_ZERO_OK)."""
    d, graphs, (ref_raw, ref_cnt, ref_tp) = large_pedigree_graphs()
    with api.Context(api.Problem.from_arrays(d), n_chains=1, lod_precision=api.SL_LOD_FP32_RESCALED,
                     lod_kernel=kernel, lod_flags=api.SL_LOD_ZERO_OK) as ctx:
        ctx.lod_score_graphs(graphs)
        raw, cnt, tp = ctx.lod_results()
    assert cnt == ref_cnt
    err = np.abs(api.lod_table(raw, cnt, tp) - api.lod_table(ref_raw, ref_cnt, ref_tp)).max()
    assert err <= FP32_LOD_TOL, err


def test_zero_trait_likelihood_policy():
    """The third graph of the set has two positions whose FP64 trait
    likelihood, peeled without rescaling as the reference does, underflows to
    0.  The plain FP64 scorer reports SL_EZERO by default (the reference exits
    there, peeler.cc:89-92) and the context stays usable; with SL_LOD_ZERO_OK
    its table equals the oracle's with those positions counted as zero terms.
    The FP32 scorer rescales every rfunction, does not underflow, and scores
    the graph without error."""
    d, graphs, (ref_raw, ref_cnt, ref_tp) = large_pedigree_graphs()
    P = port.Port(d)
    bad = graphs[2:3]
    with pytest.raises(RuntimeError):
        P.lod(bad)
    prob = api.Problem.from_arrays(d)
    with api.Context(prob, n_chains=1, lod_precision=api.SL_LOD_FP64) as ctx:
        with pytest.raises(api.SwiftLinkError) as e:
            ctx.lod_score_graphs(bad)
        assert e.value.code == api.SL_EZERO
        ctx.lod_reset()
        ctx.lod_score_graphs(graphs[:1])
        raw, cnt, tp = ctx.lod_results()
    want_raw, want_cnt, want_tp = P.lod(graphs[:1])
    assert np.abs(api.lod_table(raw, cnt, tp) - api.lod_table(want_raw, want_cnt, want_tp)).max() <= FP64_LOD_TOL
    with api.Context(prob, n_chains=1, lod_precision=api.SL_LOD_FP64, lod_flags=api.SL_LOD_ZERO_OK) as ctx:
        ctx.lod_score_graphs(graphs)
        raw, cnt, tp = ctx.lod_results()
    assert cnt == ref_cnt
    assert np.abs(api.lod_table(raw, cnt, tp) - api.lod_table(ref_raw, ref_cnt, ref_tp)).max() <= FP64_LOD_TOL
    with api.Context(prob, n_chains=1, lod_precision=api.SL_LOD_FP32_RESCALED) as ctx:
        ctx.lod_score_graphs(bad)
        raw32, _, _ = ctx.lod_results()
    assert np.all(np.isfinite(raw32)) and raw32.min() > -1e300


@pytest.mark.parametrize("name", CASES)
def test_fp64_rescaled_lod_equals_plain(name):
    """The FP64 peel with per-rfunction rescaling (for pedigrees whose unscaled
    likelihood underflows) equals the plain FP64 peel where that does not
    underflow."""
    g = load_golden(name)
    with make_ctx(g, precision=api.SL_LOD_FP64_RESCALED) as ctx:
        ctx.lod_score_graphs(g["lod_graphs"])
        raw, cnt, tp = ctx.lod_results()
    want = api.lod_table(g["lod_raw"], g["lod_count"], g["lod_trait_prob"])
    assert np.abs(api.lod_table(raw, cnt, tp) - want).max() <= FP64_LOD_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["loop", "east", "cfg1"])
def test_specialised_lsampler_is_bit_identical(name):
    """The L-sampler compiled for the pedigree (operations as constants) and
    the generic one perform the same rounded FP32 operations in the same
    order: on the same graphs and draws, explicit or from the Philox stream,
    they leave bit-identical graphs."""
    g = load_golden(name)
    C = 3
    u = np.random.default_rng(23).random((C, g["M"], g["K"] + 2 * g["N"]))
    out = {}
    for lk in LS_FORMS:
        with api.Context(api.Problem.from_arrays(g), n_chains=C, sampler_precision=api.SL_SAMPLER_FAST,
                         ls_kernel=lk) as ctx:
            assert ctx.ls_kernel_info()[0] == (lk if lk == api.SL_LS_KERNEL_SPECIALISED else api.SL_LS_KERNEL_GENERIC)
            ctx.set_graphs(np.stack([g["dg0"]] * C))
            ctx.lsampler_sweep(u, 0, C)
            swept = ctx.get_graphs()
            ctx.run(iterations=12, burnin=0, period=4, lprob=1.0, seed=9)
            out[lk] = (swept, ctx.get_graphs())
    b = out[api.SL_LS_KERNEL_SPECIALISED]
    for lk in LS_FORMS:
        assert np.array_equal(out[lk][0], b[0]), lk
        assert np.array_equal(out[lk][1], b[1]), lk


# the L-sampler's forms: generic with lanes per task by timing, forced to 32,
# 16 or 8 lanes (one, two or four tasks per warp), and the kernel specialised
# to the pedigree
LS_FORMS = (api.SL_LS_KERNEL_GENERIC, api.SL_LS_KERNEL_GENERIC32, api.SL_LS_KERNEL_GENERIC16,
            api.SL_LS_KERNEL_GENERIC8, api.SL_LS_KERNEL_SPECIALISED)


@pytest.mark.gpu
@pytest.mark.parametrize("lanes", [api.SL_LS_KERNEL_GENERIC32, api.SL_LS_KERNEL_GENERIC16,
                                   api.SL_LS_KERNEL_GENERIC8])
@pytest.mark.parametrize("name", CASES)
def test_lsweep_bit_exact_every_lane_group(name, lanes):
    """Exact mode with 32 and with 16 lanes per (chain, locus) task: the
    reference's L-sweep bit for bit (two chains, so a warp holds both tasks
    of the 16-lane form)."""
    g = load_golden(name)
    with api.Context(api.Problem.from_arrays(g), n_chains=2, ls_kernel=lanes) as ctx:
        ctx.set_graphs(np.stack([g["dg0"]] * 2))
        ctx.lsampler_sweep(np.stack([g["lsweep_u"]] * 2), 0, 2)
        out = ctx.get_graphs()
    assert np.array_equal(out[0], g["lsweep_after"])
    assert np.array_equal(out[1], g["lsweep_after"])


@pytest.mark.gpu
def test_specialised_lsampler_shared_shapes_is_bit_identical():
    """Above 150 operations the compiled L-sampler shares one function among
    operations of the same shape and passes their values in; it too leaves the
    generic kernel's graphs bit for bit (a 170-member synthetic pedigree)."""
    from swiftlink_gb300 import pedigree, synth
    spec = synth.WorkloadSpec(n_members=170, generations=5, loops=3, affected=20, markers=60, spacing_cm=0.5,
                              maf=(0.05, 0.5), missing_all=0.05)
    d = pedigree.problem_from_workload(synth.make_workload(3, seed=77, spec=spec))
    assert d["K"] > 150
    C = 4
    out = {}
    for lk in LS_FORMS:
        with api.Context(api.Problem.from_arrays(d, with_legal=False), n_chains=C,
                         sampler_precision=api.SL_SAMPLER_FAST, ls_kernel=lk) as ctx:
            ctx.set_graphs(np.stack([d["dg0"]] * C))
            ctx.run(iterations=8, burnin=0, period=4, lprob=1.0, seed=5)
            out[lk] = ctx.get_graphs()
    for lk in LS_FORMS:
        assert np.array_equal(out[lk], out[api.SL_LS_KERNEL_SPECIALISED]), lk
