"""Batches of contexts run by one graph launch per spurt (sl_batch_*).

A batch launches, for every context, the same per-chain kernels with the same
Philox streams as the context's own sl_run, so each context's graphs, LOD
table and MC3 statistics after a batch run equal those of running the
contexts one by one.  The uneven synthetic batch (pedigrees of 20-150
members with their own host-built peel sequences) runs in the fast mode and
leaves every chain with a legal graph.
"""
import numpy as np
import pytest

from conftest import load_golden
from swiftlink_gb300 import api

pytestmark = pytest.mark.gpu

RUN = dict(iterations=6, burnin=1, period=2, lprob=0.5, seed=123)


def contexts(names, temps=None):
    out = []
    for name in names:
        g = load_golden(name)
        ctx = api.Context(api.Problem.from_arrays(g), n_chains=3)
        if temps:
            ctx.set_temperatures(temps)
        ctx.set_graphs(np.stack([g["dg0"]] * 3))
        out.append(ctx)
    return out


@pytest.mark.parametrize("mc3", [False, True])
def test_batch_equals_separate_runs(mc3):
    names = ["loop", "east", "cfg1"]
    temps = [1.0, 0.8, 0.6] if mc3 else None
    ex = 2 if mc3 else 0
    solo = contexts(names, temps)
    for c in solo:
        c.run(exchange_period=ex, **RUN)
        c.synchronize()
    together = contexts(names, temps)
    with api.Batch(together) as b:
        b.run(exchange_period=ex, **RUN)
    for a, c in zip(solo, together):
        c.synchronize()
        assert np.array_equal(a.get_graphs(), c.get_graphs())
        ra, na, ta = a.lod_results()
        rc, nc, tc = c.lod_results()
        assert na == nc and ta == tc
        assert np.abs(api.lod_table(ra, na, ta) - api.lod_table(rc, nc, tc)).max() <= 1e-12
        if mc3:
            for x, y in zip(a.mc3_stats(), c.mc3_stats()):
                np.testing.assert_array_equal(x, y)
    for c in solo + together:
        c.close()


def test_uneven_synthetic_batch_fast_mode():
    from swiftlink_gb300 import pedigree, synth
    probs = [pedigree.problem_from_workload(w) for w in synth.uneven_batch(6, markers=300)]
    temps = [0.3 ** (j / 3) for j in range(4)]
    ctxs = []
    for d in probs:
        ctx = api.Context(api.Problem.from_arrays(d, with_legal=False), n_chains=4,
                          lod_precision=api.SL_LOD_FP32_RESCALED, sampler_precision=api.SL_SAMPLER_FAST,
                          lod_flags=api.SL_LOD_ZERO_OK)
        ctx.set_temperatures(temps)
        ctx.set_graphs(np.stack([d["dg0"]] * 4))
        ctxs.append(ctx)
    with api.Batch(ctxs) as b:
        b.run(iterations=20, burnin=5, period=5, lprob=0.5, seed=9, exchange_period=5)
    for ctx in ctxs:
        ctx.synchronize()
        for c in range(4):
            assert ctx.chain_loglik(c, c) > -1e300
        raw, cnt, tp = ctx.lod_results()
        assert cnt == 4                      # the t = 1 chain, iterations 5, 10, 15, 20 - 1
        assert np.isfinite(api.lod_table(raw, cnt, tp)).all()
        acc, prop = ctx.mc3_stats()
        assert prop.sum() == 5
        ctx.close()
