"""Sequential imputation: legal starting graphs on the device.

One pass (LocusSampler::start_from, locus_sampler2.cc:214-241) visits the
start locus with neither neighbour, then the loci to its left with only the
right neighbour, then those to its right with only the left neighbour, each a
full L-sampler step; the weight is the sum of the log peel results.  The
oracle's pass equals the reference's own (same start, same draws) bit for bit;
the device pass (exact mode) equals the oracle's; in the FP32 mode (every
rfunction rescaled by a power of two) the weights keep the removed exponents,
so they match the oracle's to FP32 accuracy; the Philox-driven best-of-n run
leaves every chain with a legal graph.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import port, ref
from swiftlink_gb300 import api

needs_ref = pytest.mark.skipif(not ref.available(), reason="reference build not present")


@needs_ref
def test_oracle_pass_equals_reference(tmp_path):
    import dataclasses
    from swiftlink_gb300 import synth
    paths = synth.workload_files(1, str(tmp_path))
    r = ref.Ref(*paths, n_lod=5, peel_iters=10000, seed=1)
    P = port.Port(dataclasses.asdict(r.problem()))
    rng = np.random.default_rng(6)
    for start in (0, 91, r.M - 1):
        u = rng.random(40000)
        dg0 = np.zeros((r.M, r.N, 2), np.int32)
        a, na, wa = r.si(dg0, start, u)
        b, nb, wb = P.si(dg0, start, u)
        assert na == nb and wa == wb and np.array_equal(a, b)
    r.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["loop", "east", "cfg1"])
def test_device_pass_equals_oracle(name):
    g = load_golden(name)
    P = port.Port(g)
    C = 3
    rng = np.random.default_rng(7)
    starts = np.array([0, g["M"] // 2, g["M"] - 1], np.int32)
    L = g["M"] * (g["K"] + 2 * g["N"])
    u = rng.random((C, L))
    with api.Context(api.Problem.from_arrays(g), n_chains=C) as ctx:
        ctx.set_graphs(np.zeros((C, g["M"], g["N"], 2), np.int32))
        w = ctx.sequential_imputation(starts, u)
        out = ctx.get_graphs()
    for c in range(C):
        dg, _, want_w = P.si(np.zeros((g["M"], g["N"], 2), np.int32), int(starts[c]), u[c])
        assert np.array_equal(out[c], dg), c
        assert abs(w[c] - want_w) <= 1e-12 * abs(want_w)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["east", "cfg1"])
def test_fast_pass_weights_match_oracle(name):
    """The FP32 pass's weights against the FP64 pass's on the same start
    loci and draws: equal to FP32 accuracy where both drew the same graph, of
    the same magnitude where a near-tie drew differently.  Rescaled
    rfunctions would leave the FP32 weights short by every removed exponent
    (tens of natural-log units per locus)."""
    g = load_golden(name)
    C = 3
    rng = np.random.default_rng(8)
    starts = np.array([0, g["M"] // 2, g["M"] - 1], np.int32)
    L = g["M"] * (g["K"] + 2 * g["N"])
    u = rng.random((C, L))
    out = {}
    for prec in (api.SL_SAMPLER_EXACT, api.SL_SAMPLER_FAST):
        with api.Context(api.Problem.from_arrays(g), n_chains=C, sampler_precision=prec) as ctx:
            ctx.set_graphs(np.zeros((C, g["M"], g["N"], 2), np.int32))
            w = ctx.sequential_imputation(starts, u)
            out[prec] = (w, ctx.get_graphs())
    we, ge = out[api.SL_SAMPLER_EXACT]
    wf, gf = out[api.SL_SAMPLER_FAST]
    for c in range(C):
        if np.array_equal(ge[c], gf[c]):   # same graph: same weight up to FP32 rounding
            assert abs(wf[c] - we[c]) <= 1e-4 * abs(we[c]) + 1e-3, (c, wf[c], we[c])
        else:                              # a near-tie drew differently: same order of magnitude
            assert abs(wf[c] - we[c]) <= 0.05 * abs(we[c]), (c, wf[c], we[c])


@pytest.mark.gpu
@pytest.mark.parametrize("fast", [False, True])
def test_best_of_n_imputation_gives_legal_graphs(fast):
    g = load_golden("cfg1")
    P = port.Port(g)
    C = 4
    prec = api.SL_SAMPLER_FAST if fast else api.SL_SAMPLER_EXACT
    with api.Context(api.Problem.from_arrays(g), n_chains=C, sampler_precision=prec) as ctx:
        best = ctx.sequential_imputation_run(iterations=5, seed=11)
        out = ctx.get_graphs()
    for c in range(C):
        ll = P.loglik(out[c])
        assert ll > -1e300
        assert np.isfinite(best[c])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["east", "cfg1"])
def test_batched_best_of_n_equals_pass_by_pass(name):
    """sl_sequential_imputation_run runs its passes as one batch of
    independent warps; replaying each pass alone (sl_sequential_imputation
    with the same start loci and the same Philox draws) and keeping the first
    strictly better weight gives the same graphs and weights."""
    from swiftlink_gb300 import philox as ph
    g = load_golden(name)
    C, n, seed = 3, 6, 4242
    M = g["M"]
    L = M * (g["K"] + 2 * g["N"])
    with api.Context(api.Problem.from_arrays(g), n_chains=C) as ctx:
        best = ctx.sequential_imputation_run(iterations=n, seed=seed)
        batched = ctx.get_graphs()
    want_w = np.full(C, -np.finfo(np.float64).max)
    want_g = [None] * C
    with api.Context(api.Problem.from_arrays(g), n_chains=C) as ctx:
        for p in range(n):
            starts = np.array([min(M - 1, int(ph.uniform(seed, ph.stage_hi(c, p, 6), 0) * M)) for c in range(C)],
                              np.int32)
            u = np.stack([ph.uniform(seed, ph.stage_hi(c, p, 5), np.arange(L, dtype=np.uint64)) for c in range(C)])
            ctx.set_graphs(np.zeros((C, M, g["N"], 2), np.int32))
            w = ctx.sequential_imputation(starts, u)
            out = ctx.get_graphs()
            for c in range(C):
                if w[c] > want_w[c]:
                    want_w[c], want_g[c] = w[c], out[c].copy()
    np.testing.assert_array_equal(best, want_w)
    for c in range(C):
        assert np.array_equal(batched[c], want_g[c]), c
