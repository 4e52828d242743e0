"""Parity on the largest single-GPU workload: the seeded 400-member,
8-generation, 10-loop pedigree with 10,000 SNPs at 0.1 cM (87 founders,
400 peel operations, cutsets up to 5 members).

* Exact-mode L-steps at 20 spread loci and an exact-mode M-sweep over 8
  meioses, bit-exact against the C restatement of the reference with the same
  uniforms.
* LOD scores of two graphs: the reference's plain FP64 peel underflows at
  every position of this pedigree (Peeler::process then stops,
  peeler.cc:89-92), so the checker is the restatement's FP64 peel with
  per-rfunction power-of-two rescaling, itself pinned to the reference's
  plain peel where that does not underflow (tests/test_oracle_pin.py).  The
  device's FP64-rescaled form must agree within |dLOD| <= 1e-10, the batched
  FP32-rescaled forms within |dLOD| <= 1e-3, on a 300-interval slice (1,500
  positions per graph) that the checker scores in about a second.
"""
import ctypes

import numpy as np
import pytest

from oracle import port
from swiftlink_gb300 import api, pedigree, synth

pytestmark = pytest.mark.gpu

SLICE = (4000, 4300)


def _legal(d):
    desc = api.Problem.from_arrays(d, with_legal=False).desc()
    out = np.zeros((d["M"], d["N"]), np.uint8)
    assert api.lib().sl_problem_legal_masks(ctypes.byref(desc), out.ctypes.data_as(ctypes.c_void_p)) == 0
    return out


@pytest.fixture(scope="module")
def cfg5():
    port.build()
    d = pedigree.problem_from_workload(synth.make_workload(5))
    d["legal"] = _legal(d)
    d["trait_prior"] = port.derive_priors(d["genotypes"], d["typed"], d["minor"])
    assert (d["N"], d["M"]) == (400, 10000)
    return d, port.Port(d)


@pytest.mark.parametrize("lanes", [api.SL_LS_KERNEL_GENERIC32, api.SL_LS_KERNEL_GENERIC16,
                                   api.SL_LS_KERNEL_GENERIC8])
def test_cfg5_exact_lsteps_bit_exact(cfg5, lanes):
    d, P = cfg5
    M, K, N = d["M"], d["K"], d["N"]
    loci = np.array([0, M - 1] + [250 + 500 * i + (i % 2) for i in range(18)], np.int32)
    rng = np.random.default_rng(51)
    u = np.zeros((1, M, K + 2 * N))
    u[0, loci] = rng.random((loci.size, K + 2 * N))
    with api.Context(api.Problem.from_arrays(d), n_chains=1, ls_kernel=lanes) as ctx:
        assert np.array_equal(ctx.trait_priors(), d["trait_prior"])
        ctx.set_graphs(d["dg0"][None])
        ctx.lsampler_loci(loci, u)
        got = ctx.get_graphs()[0]
    want = d["dg0"].copy()
    for l in loci:
        want, _ = P.lstep(want, int(l), u[0, l])
    assert np.array_equal(got, want)
    assert not np.array_equal(want, d["dg0"])   # the steps changed the graph


def test_cfg5_exact_msweep_bit_exact(cfg5):
    d, P = cfg5
    rng = np.random.default_rng(52)
    order = d["meioses"].copy()
    rng.shuffle(order)
    order = order[:8]
    u = rng.random((1, order.size, d["M"]))
    with api.Context(api.Problem.from_arrays(d), n_chains=1) as ctx:
        ctx.set_graphs(d["dg0"][None])
        ctx.msampler_sweep(order, u)
        got = ctx.get_graphs()[0]
    want, _ = P.msweep(d["dg0"], order, u[0])
    assert np.array_equal(got, want)
    assert not np.array_equal(want, d["dg0"])


@pytest.fixture(scope="module")
def cfg5_lod(cfg5):
    """Two legal graphs (the gene drop's and an M-swept one) and the checker's
    rescaled FP64 log-sums, count and log P(T) on the slice."""
    d, P = cfg5
    rng = np.random.default_rng(53)
    order = d["meioses"].copy()
    rng.shuffle(order)
    g1, _ = P.msweep(d["dg0"], order[:16], rng.random((16, d["M"])))
    graphs = np.stack([d["dg0"], g1])
    raw, cnt, tp = P.lod_range(graphs, SLICE[0], SLICE[1], rescale=True)
    assert (raw > -1e300).all()
    return graphs, api.lod_table(raw, cnt, tp)


@pytest.mark.parametrize("prec,kernel,tol", [
    (api.SL_LOD_FP64_RESCALED, api.SL_LOD_KERNEL_AUTO, 1e-10),
    (api.SL_LOD_FP32_RESCALED, api.SL_LOD_KERNEL_AUTO, 1e-3),
    (api.SL_LOD_FP32_RESCALED, api.SL_LOD_KERNEL_INTERP, 1e-3),
])
def test_cfg5_lod_against_rescaled_oracle(cfg5, cfg5_lod, prec, kernel, tol):
    """Also: no position's FP32 likelihood underflows (the default flags make
    a zero likelihood an error)."""
    d, _ = cfg5
    graphs, want = cfg5_lod
    n = d["n_lod"]
    with api.Context(api.Problem.from_arrays(d, with_legal=False), n_chains=2, lod_precision=prec,
                     lod_kernel=kernel) as ctx:
        ctx.lod_score_graphs(graphs)
        raw, cnt, tp = ctx.lod_results()
    assert cnt == 2
    assert (raw > -1e300).all()
    got = api.lod_table(raw, cnt, tp)[SLICE[0] * n:SLICE[1] * n]
    err = float(np.abs(got - want).max())
    assert err <= tol, err


def test_cfg5_plain_fp64_underflows_as_the_reference(cfg5, cfg5_lod):
    """The plain FP64 form (the reference's arithmetic) finds a zero trait
    likelihood at every position and reports it, as Peeler::process stops
    there."""
    d, _ = cfg5
    graphs, _ = cfg5_lod
    with api.Context(api.Problem.from_arrays(d, with_legal=False), n_chains=1) as ctx:
        with pytest.raises(api.SwiftLinkError) as e:
            ctx.lod_score_graphs(graphs[:1])
            ctx.synchronize()
        assert e.value.code == api.SL_EZERO
