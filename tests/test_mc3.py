"""MC3: tempered chains and the exchange of adjacent chains' graphs.

A chain at temperature t samples under theta_t = (t theta) + ((1 - t) 0.5)
and maf_t likewise (GeneticMap::set_temperature, genetic_map.cc:95-117); its
L-sampler priors stay those of temperature 1 (cached while parsing,
pedigree_parser.cc:157).  Every spurt of `exchange_period` iterations ends with
one proposed exchange between a uniformly chosen adjacent pair, accepted with
probability min(1, exp((xy + yx) - (xx + yy))) from the four log-likelihoods of
DescentGraph::get_likelihood2 (mc3.cc:117-158).  Only chains at t = 1 are
scored (markov_chain.cc:173-174).

CPU: the oracle's tempered sampler steps and log-likelihood against the
reference's own (tempered map, same uniforms), bit for bit.  GPU: tempered
sweeps, chain log-likelihoods and a device-driven MC3 run against the oracle.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import port, ref
from swiftlink_gb300 import api
from swiftlink_gb300 import philox as philox_np

FP64_LOD_TOL = 1e-10
TEMPS = [1.0, 0.8, 0.6]

needs_ref = pytest.mark.skipif(not ref.available(), reason="reference build not present")


def test_port_loglik_equals_golden_bitwise():
    for name in ("loop", "east", "cfg1"):
        g = load_golden(name)
        assert port.Port(g).loglik(g["dg0"]) == g["loglik0"], name


@needs_ref
@pytest.mark.parametrize("t", [0.75, 0.4])
def test_tempered_oracle_matches_reference(t, tmp_path):
    import dataclasses
    from swiftlink_gb300 import synth
    paths = synth.workload_files(1, str(tmp_path))
    r = ref.Ref(*paths, n_lod=5, peel_iters=10000, seed=1)
    p = dataclasses.asdict(r.problem())
    dg, _ = r.initial_dg(2)
    assert r.loglik_tempered(dg, t) == port.Port(port.tempered(p, t)).loglik(dg)
    r.set_temperature(t)
    P = port.Port(port.tempered(p, t))
    rng = np.random.default_rng(int(t * 100))
    stride = r.K + 2 * r.N
    for l in rng.choice(r.M, size=30, replace=False):
        u = rng.random(stride)
        a, na = r.lstep(dg, int(l), u)
        b, nb = P.lstep(dg, int(l), u)
        assert na == nb and np.array_equal(a, b)
        dg = a
    order = p["meioses"].copy()
    rng.shuffle(order)
    order = order[:10]
    u = rng.random((order.size, r.M))
    a, ua = r.msweep(dg, order, u)
    b, ub = P.msweep(dg, order, u)
    assert np.array_equal(a, b) and np.array_equal(ua, ub)
    r.close()


# ----------------------------------------------------------------- GPU ----

@pytest.mark.gpu
@pytest.mark.parametrize("name", ["loop", "cfg1"])
def test_tempered_sweeps_bit_exact(name):
    g = load_golden(name)
    C = len(TEMPS)
    rng = np.random.default_rng(5)
    st = g["K"] + 2 * g["N"]
    ul = rng.random((C, g["M"], st))
    order = g["msweep_order"]
    um = rng.random((C, order.size, g["M"]))
    with api.Context(api.Problem.from_arrays(g), n_chains=C) as ctx:
        ctx.set_temperatures(TEMPS)
        ctx.set_graphs(np.stack([g["dg0"]] * C))
        ctx.lsampler_sweep(ul, n_chains=C)
        ctx.msampler_sweep(order, um, n_chains=C)
        out = ctx.get_graphs()
        ll = [[ctx.chain_loglik(a, b) for b in range(C)] for a in range(C)]
    for c, t in enumerate(TEMPS):
        P = port.Port(port.tempered(g, t))
        dg = g["dg0"].copy()
        for l in list(range(0, g["M"], 2)) + list(range(1, g["M"], 2)):
            dg, _ = P.lstep(dg, l, ul[c, l])
        dg, _ = P.msweep(dg, order, um[c])
        assert np.array_equal(out[c], dg), f"chain {c} (t = {t})"
    for a in range(C):
        for b in range(C):
            want = port.Port(port.tempered(g, TEMPS[b])).loglik(out[a])
            assert ll[a][b] == want, (a, b, ll[a][b], want)


def replay_mc3(g, temps, dg0, seed, iters, lprob, period, burnin, exchange):
    """Host replay of an MC3 run: per chain the run's schedule under its
    tempered map, an exchange after every full spurt."""
    M, K, N = g["M"], g["K"], g["N"]
    st = K + 2 * N
    base = g["meioses"]
    C = len(temps)
    Ps = [port.Port(port.tempered(g, t)) for t in temps]
    dgs = [dg0.copy() for _ in range(C)]
    scored, swaps = [], []
    total = iters + burnin
    for it0 in range(0, total, exchange):
        it1 = min(total, it0 + exchange)
        for it in range(it0, it1):
            for c in range(C):
                P = Ps[c]
                if philox_np.chooses_l(seed, c, it, lprob):
                    u = philox_np.lsweep_draws(seed, c, it, M, st)
                    for l in list(range(0, M, 2)) + list(range(1, M, 2)):
                        dgs[c], _ = P.lstep(dgs[c], l, u[l])
                else:
                    order = philox_np.shuffled(seed, c, it, base)
                    u = philox_np.msweep_draws(seed, c, it, order.size, M)
                    dgs[c], _ = P.msweep(dgs[c], order, u)
            if it >= burnin and it % period == 0:
                scored.extend(dgs[c].copy() for c in range(C) if temps[c] == 1.0)
        if it1 - it0 == exchange:
            u0, u1 = philox_np.exchange_draws(seed, it1)
            r = min(int((C - 1) * u0), C - 2)
            xx = Ps[r].loglik(dgs[r])
            yy = Ps[r + 1].loglik(dgs[r + 1])
            xy = Ps[r].loglik(dgs[r + 1])
            yx = Ps[r + 1].loglik(dgs[r])
            ratio = (xy + yx) - (xx + yy)
            acc = u1 == 0.0 or np.log(u1) < min(0.0, ratio)
            if acc:
                dgs[r], dgs[r + 1] = dgs[r + 1], dgs[r]
            swaps.append((r, acc))
    return dgs, scored, swaps


# near-equal temperatures: the exchange ratio is close to 0, so most
# proposed exchanges must be accepted (and are checked one by one)
CLOSE_TEMPS = [1.0, 0.9995, 0.999]


@pytest.mark.gpu
@pytest.mark.parametrize("temps", [TEMPS, CLOSE_TEMPS], ids=["spread", "close"])
@pytest.mark.parametrize("name", ["loop", "cfg1"])
def test_mc3_run_matches_host_replay(name, temps):
    g = load_golden(name)
    TEMPS = temps
    C, seed, iters, burnin, period, exchange = len(TEMPS), 77, 8, 2, 2, 2
    with api.Context(api.Problem.from_arrays(g), n_chains=C) as ctx:
        ctx.set_temperatures(TEMPS)
        ctx.set_graphs(np.stack([g["dg0"]] * C))
        ctx.run(iterations=iters, burnin=burnin, period=period, lprob=0.5, seed=seed, exchange_period=exchange)
        ctx.synchronize()
        out = ctx.get_graphs()
        raw, cnt, tp = ctx.lod_results()
        acc, prop = ctx.mc3_stats()
    dgs, scored, swaps = replay_mc3(g, TEMPS, g["dg0"], seed, iters, 0.5, period, burnin, exchange)
    for c in range(C):
        assert np.array_equal(out[c], dgs[c]), f"chain {c}"
    want_prop = np.bincount([r for r, _ in swaps], minlength=C - 1)
    want_acc = np.bincount([r for r, a in swaps if a], minlength=C - 1)
    np.testing.assert_array_equal(prop, want_prop)
    np.testing.assert_array_equal(acc, want_acc)
    if temps is CLOSE_TEMPS:
        assert acc.sum() >= prop.sum() // 2 and acc.sum() > 0, (acc, prop)
    P = port.Port(g)
    ref_raw, ref_cnt, ref_tp = P.lod(np.stack(scored))
    assert cnt == ref_cnt
    assert np.abs(api.lod_table(raw, cnt, tp) - api.lod_table(ref_raw, ref_cnt, ref_tp)).max() <= FP64_LOD_TOL


@pytest.mark.gpu
def test_temperatures_are_validated():
    g = load_golden("loop")
    with api.Context(api.Problem.from_arrays(g), n_chains=2) as ctx:
        with pytest.raises(api.SwiftLinkError):
            ctx.set_temperatures([1.0, 0.0])
        with pytest.raises(api.SwiftLinkError):
            ctx.set_temperatures([1.0, 1.5])


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_split_run_exchanges_as_one_run(batched):
    """Exchanges follow multiples of the exchange period counted from iteration
    0, so a run resumed at any first_iteration is the unbroken run."""
    g = load_golden("cfg1")
    C, seed, iters, burnin, period, exchange = len(TEMPS), 91, 20, 4, 2, 3
    outs = []
    for splits in ([], [5, 11, 12]):
        with api.Context(api.Problem.from_arrays(g), n_chains=C) as ctx:
            ctx.set_temperatures(TEMPS)
            ctx.set_graphs(np.stack([g["dg0"]] * C))
            runner = api.Batch([ctx]) if batched else ctx
            total = iters + burnin
            bounds = [0] + splits + [total]
            for a, b in zip(bounds[:-1], bounds[1:]):
                runner.run(iterations=b - burnin if b > burnin else 0, burnin=burnin if b > burnin else b,
                           period=period, lprob=0.5, seed=seed, first_iteration=a, exchange_period=exchange)
            ctx.synchronize()
            outs.append((ctx.get_graphs(), ctx.lod_results(), ctx.mc3_stats()))
            if batched:
                runner.close()
    (g0, l0, s0), (g1, l1, s1) = outs
    assert np.array_equal(g0, g1)
    np.testing.assert_array_equal(l0[0], l1[0])
    assert l0[1] == l1[1] and l0[2] == l1[2]
    np.testing.assert_array_equal(s0[0], s1[0])
    np.testing.assert_array_equal(s0[1], s1[1])
    assert s0[1].sum() == total // exchange


@pytest.mark.gpu
def test_persistent_mc3_graph_equals_host_driven_spurts():
    """An MC3 run is one launch of a graph whose outer loop runs every spurt and
    its exchange on the device; with per-kernel profiling on, the same spurts
    and exchanges are launched one by one from the host.  Both give the same
    graphs, scores and exchange counts."""
    g = load_golden("cfg1")
    C, seed, iters, burnin, period, exchange = 4, 13, 30, 5, 5, 4
    temps = [1.0, 0.999, 0.998, 0.997]
    outs = []
    for profiled in (False, True):
        with api.Context(api.Problem.from_arrays(g), n_chains=C, sampler_precision=api.SL_SAMPLER_FAST,
                         lod_precision=api.SL_LOD_FP32_RESCALED, lod_flags=api.SL_LOD_ZERO_OK) as ctx:
            ctx.set_temperatures(temps)
            ctx.set_graphs(np.stack([g["dg0"]] * C))
            ctx.profile(profiled)
            ctx.run(iterations=iters, burnin=burnin, period=period, lprob=0.5, seed=seed, exchange_period=exchange)
            ctx.synchronize()
            outs.append((ctx.get_graphs(), ctx.lod_results(), ctx.mc3_stats()))
    (g0, l0, s0), (g1, l1, s1) = outs
    assert np.array_equal(g0, g1)
    # the same graphs scored; the one-by-one path merges each scoring's graphs
    # as it goes and may time the FP32 scorer's forms, so the log-sums agree to
    # FP32 rounding rather than bit for bit
    np.testing.assert_allclose(l0[0], l1[0], rtol=0, atol=1e-5)
    assert l0[1] == l1[1]
    np.testing.assert_array_equal(s0[0], s1[0])
    np.testing.assert_array_equal(s0[1], s1[1])
    assert s0[1].sum() == (iters + burnin) // exchange
    assert s0[0].sum() > 0   # near-equal temperatures: exchanges are accepted
