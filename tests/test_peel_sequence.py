"""The host peel-sequence generator (sl_peel_sequence) and the host problem
builder (swiftlink_gb300/pedigree.py).

A peel sequence only orders the work: any legal sequence gives the same
trait likelihoods, so the generated sequences are checked against the
reference's own sequences of the golden cases through the oracle (P(T) and
every LOD position, FP64), for structure (each member peeled once, every
function consumed once, LAST at the end), and on the GPU for bit-exact sweeps
against the oracle running the same sequence.
"""
import numpy as np
import pytest

from conftest import CASES, load_golden
from oracle import port
from swiftlink_gb300 import api


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()


def with_generated_ops(g):
    ot, op, cut, prev, ch = api.peel_sequence(g["mother"], g["father"])
    return dict(g, op_type=ot, op_peel=op, op_cutset=cut, op_prev=prev, op_children=ch, K=len(ot))


@pytest.mark.parametrize("name", CASES)
def test_generated_sequence_gives_the_reference_likelihoods(name):
    g = load_golden(name)
    d = with_generated_ops(g)
    graphs = g["lod_graphs"]
    r1 = port.Port(g).lod(graphs)
    r2 = port.Port(d).lod(graphs)
    assert abs(r1[2] - r2[2]) <= 1e-12 * abs(r1[2])
    np.testing.assert_allclose(r2[0], r1[0], rtol=0, atol=1e-9)
    # and no worse than the reference's search by its own cost (sum of cutset sizes)
    assert sum(len(c) for c in d["op_cutset"]) <= sum(len(c) for c in g["op_cutset"]) + 2


@pytest.mark.parametrize("name", CASES)
def test_generated_sequence_structure(name):
    g = load_golden(name)
    d = with_generated_ops(g)
    N = g["N"]
    assert sorted(d["op_peel"].tolist()) == list(range(N))
    assert d["op_type"][-1] == 4 and (d["op_type"][:-1] != 4).all()   # LAST_PEEL only at the end
    used = np.concatenate([p for p in d["op_prev"] if len(p)] or [np.zeros(0, np.int32)])
    assert sorted(used.tolist()) == list(range(N - 1))               # every function consumed once
    for k, prevs in enumerate(d["op_prev"]):
        assert all(p < k for p in prevs)
    for k in range(N):
        if d["op_type"][k] == 2:                                      # PARENT_PEEL: children are offspring
            kids = [i for i in range(N) if g["mother"][i] == d["op_peel"][k] or g["father"][i] == d["op_peel"][k]]
            assert all(c in kids for c in d["op_children"][k]) and len(d["op_children"][k]) > 0


def test_problem_from_synthetic_workload():
    """The host builder on the 30-member workload: the same pedigree, genotypes
    and model as the reference build of the same files (up to the order of
    members), the same P(T), and the gene drop's graph is legal."""
    from swiftlink_gb300 import pedigree, synth
    g = load_golden("cfg1")
    d = pedigree.problem_from_workload(synth.make_workload(1))
    assert (d["N"], d["F"], d["M"]) == (g["N"], g["F"], g["M"])
    assert sorted(np.bincount(d["genotypes"].ravel(), minlength=4)) == sorted(
        np.bincount(g["genotypes"].ravel(), minlength=4))
    np.testing.assert_allclose(d["theta"], g["theta"], rtol=1e-12)
    np.testing.assert_allclose(d["partial"], g["partial"], rtol=1e-12)
    np.testing.assert_allclose(d["minor"], g["minor"], atol=1e-10)      # the DAT file keeps 10 decimals
    d["trait_prior"] = port.derive_priors(d["genotypes"], d["typed"], d["minor"])
    import ctypes
    prob = api.Problem.from_arrays(d, with_legal=False)
    desc = prob.desc()
    legal = np.zeros((d["M"], d["N"]), np.uint8)
    assert api.lib().sl_problem_legal_masks(ctypes.byref(desc), legal.ctypes.data_as(ctypes.c_void_p)) == 0
    d["legal"] = legal
    P = port.Port(d)
    assert P.loglik(d["dg0"]) > -1e300
    _, _, tp = P.lod(d["dg0"][None])
    assert abs(tp - g["lod_trait_prob"]) <= 1e-12 * abs(tp)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["east", "cfg1"])
def test_generated_sequence_sweeps_bit_exact(name):
    g = load_golden(name)
    d = with_generated_ops(g)
    P = port.Port(d)
    rng = np.random.default_rng(8)
    st = d["K"] + 2 * d["N"]
    u = rng.random((g["M"], st))
    order = g["msweep_order"]
    um = rng.random((order.size, g["M"]))
    with api.Context(api.Problem.from_arrays(d), n_chains=1) as ctx:
        ctx.set_graphs(g["dg0"])
        ctx.lsampler_sweep(u[None])
        ctx.msampler_sweep(order, um[None])
        out = ctx.get_graphs()[0]
        ctx.lod_score_graphs(g["lod_graphs"])
        raw, cnt, tp = ctx.lod_results()
    dg = g["dg0"].copy()
    for l in list(range(0, g["M"], 2)) + list(range(1, g["M"], 2)):
        dg, _ = P.lstep(dg, l, u[l])
    dg, _ = P.msweep(dg, order, um)
    assert np.array_equal(out, dg)
    want = P.lod(g["lod_graphs"])
    assert np.abs(api.lod_table(raw, cnt, tp) - api.lod_table(*want)).max() <= 1e-10
