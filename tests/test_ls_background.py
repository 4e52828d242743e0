"""The specialised FP32 L-sampler compiled on a host thread (SL_LS_KERNEL_BACKGROUND).

A context starts on the generic kernel and switches to the compiled one at a
run or L-sampler call after the compile ends; the two kernels draw the same
graphs, and a switch keeps the chains' pending LOD tables, so the graphs and
the LOD table of a run are bit for bit those of a run on the generic kernel
alone, wherever the switch falls.  Identical sources compile once per process.
"""
import time

import numpy as np
import pytest

from swiftlink_gb300 import api

pytestmark = pytest.mark.gpu

WAIT_S = 300.0   # the longest a compile of these small pedigrees may take


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()


def synthetic(seed, members=60, markers=80):
    """A pedigree whose generated L-sampler no other test compiles (the
    process-wide cache would otherwise hand it over at once)."""
    from swiftlink_gb300 import pedigree, synth
    spec = synth.WorkloadSpec(n_members=members, generations=4, loops=2, affected=8, markers=markers,
                              spacing_cm=0.5, maf=(0.05, 0.5), missing_all=0.05)
    return pedigree.problem_from_workload(synth.make_workload(3, seed=seed, spec=spec))


def context(d, C, lk):
    # a fixed scoring kernel: the timed choice (SL_LOD_KERNEL_AUTO) may differ between two contexts, and
    # the candidates differ in the last FP32 bits
    return api.Context(api.Problem.from_arrays(d, with_legal=False), n_chains=C,
                       sampler_precision=api.SL_SAMPLER_FAST, lod_precision=api.SL_LOD_FP32_RESCALED,
                       lod_kernel=api.SL_LOD_KERNEL_JIT_REG, ls_kernel=lk)


def wait_compiled(ctx):
    t0 = time.time()
    while time.time() - t0 < WAIT_S:
        k, ms = ctx.ls_kernel_info()
        if ms >= 0:
            return k, ms
        time.sleep(0.05)
    raise AssertionError("the background compile did not end")


def run_pieces(ctx, bounds, seed, period):
    for a, b in zip(bounds[:-1], bounds[1:]):
        ctx.run(iterations=b, burnin=0, period=period, lprob=0.5, seed=seed, first_iteration=a)


def test_background_switch_between_runs_is_bit_identical():
    d = synthetic(4242)
    C, N, period, seed = 3, 120, 5, 11
    with context(d, C, api.SL_LS_KERNEL_GENERIC) as ref:
        ref.set_graphs(np.stack([d["dg0"]] * C))
        ref.run(iterations=N, burnin=0, period=period, lprob=0.5, seed=seed)
        want_g, want_l = ref.get_graphs(), ref.lod_results()
    with context(d, C, api.SL_LS_KERNEL_BACKGROUND) as ctx:
        ctx.set_graphs(np.stack([d["dg0"]] * C))
        run_pieces(ctx, [0, 20], seed, period)
        k, ms = ctx.ls_kernel_info()
        assert (k, ms) == (api.SL_LS_KERNEL_GENERIC, -1.0)   # the first piece ran on the generic kernel
        k, ms = wait_compiled(ctx)
        assert k == api.SL_LS_KERNEL_SPECIALISED and ms > 0
        run_pieces(ctx, [20, 65, N], seed, period)   # the chains' tables hold scores from both kernels
        got_g, got_l = ctx.get_graphs(), ctx.lod_results()
    assert np.array_equal(got_g, want_g)
    assert np.array_equal(got_l[0], want_l[0]) and got_l[1:] == want_l[1:]


def test_background_long_run_is_bit_identical():
    """One sl_run call while the compile runs: spans of a few iterations, the
    switch wherever the compile ends."""
    d = synthetic(4343)
    C, N, period, seed = 2, 400, 10, 12
    with context(d, C, api.SL_LS_KERNEL_GENERIC) as ref:
        ref.set_graphs(np.stack([d["dg0"]] * C))
        ref.run(iterations=N, burnin=0, period=period, lprob=0.5, seed=seed)
        want_g, want_l = ref.get_graphs(), ref.lod_results()
    with context(d, C, api.SL_LS_KERNEL_BACKGROUND) as ctx:
        ctx.set_graphs(np.stack([d["dg0"]] * C))
        ctx.run(iterations=N, burnin=0, period=period, lprob=0.5, seed=seed)
        got_g, got_l = ctx.get_graphs(), ctx.lod_results()
        wait_compiled(ctx)
    assert np.array_equal(got_g, want_g)
    assert np.array_equal(got_l[0], want_l[0]) and got_l[1:] == want_l[1:]


def test_background_batch_is_bit_identical():
    """A batch recaptures its graph when one of its contexts switches."""
    ds = [synthetic(4444), synthetic(4545, members=40, markers=60)]
    C, N, period, seed = 2, 90, 5, 13

    def run(lk, wait_after):
        ctxs = [context(d, C, lk) for d in ds]
        try:
            for c, d in zip(ctxs, ds):
                c.set_graphs(np.stack([d["dg0"]] * C))
            with api.Batch(ctxs) as b:
                b.run(iterations=wait_after, burnin=0, period=period, lprob=0.5, seed=seed)
                if lk == api.SL_LS_KERNEL_BACKGROUND:
                    for c in ctxs:
                        assert wait_compiled(c)[0] == api.SL_LS_KERNEL_SPECIALISED
                b.run(iterations=N, burnin=0, period=period, lprob=0.5, seed=seed, first_iteration=wait_after)
            return [(c.get_graphs(), c.lod_results()) for c in ctxs]
        finally:
            for c in ctxs:
                c.close()

    want = run(api.SL_LS_KERNEL_GENERIC, 30)
    got = run(api.SL_LS_KERNEL_BACKGROUND, 30)
    for (wg, wl), (gg, gl) in zip(want, got):
        assert np.array_equal(gg, wg)
        assert np.array_equal(gl[0], wl[0]) and gl[1:] == wl[1:]


def test_identical_sources_compile_once():
    d = synthetic(4646, members=50, markers=40)
    with context(d, 2, api.SL_LS_KERNEL_SPECIALISED) as a:
        first = a.ls_kernel_info()[1]
        with context(d, 2, api.SL_LS_KERNEL_SPECIALISED) as b:
            again = b.ls_kernel_info()[1]
    assert first > 0 and again < 0.25 * first
