"""Pin the C restatement of the reference (oracle/sl_oracle.c) before trusting it.

1. Against the committed golden vectors written by the reference's own code
   (tests/golden/make_golden.py): bit-identical descent graphs after L-steps,
   an L-sweep and an M-sweep, and LOD log-sums.
2. Against the reference build itself (oracle/_ref), on freshly seeded inputs,
   where that build exists (the development container only).
"""
import os

import numpy as np
import pytest

from conftest import load_golden, CASES
from oracle import port, ref


@pytest.fixture(scope="module", autouse=True)
def _built():
    port.build()


@pytest.mark.parametrize("name", CASES)
def test_port_lsteps_match_golden(name):
    g = load_golden(name)
    P = port.Port(g)
    dg = g["dg0"].copy()
    for i, l in enumerate(g["lstep_loci"]):
        dg, used = P.lstep(dg, int(l), g["lstep_u"][i])
        assert used == g["lstep_used"][i]
        assert np.array_equal(dg, g["lstep_after"][i]), f"locus {l}"


@pytest.mark.parametrize("name", CASES)
def test_port_lsweep_matches_golden(name):
    g = load_golden(name)
    P = port.Port(g)
    dg = g["dg0"].copy()
    M = g["M"]
    for l in list(range(0, M, 2)) + list(range(1, M, 2)):
        dg, _ = P.lstep(dg, l, g["lsweep_u"][l])
    assert np.array_equal(dg, g["lsweep_after"])


@pytest.mark.parametrize("name", CASES)
def test_port_one_call_lsweep_matches_golden(name):
    """slo_lsweep (the whole even-then-odd sweep in one call, one workspace
    reused by every locus, the timed CPU arm's L-sweep) equals the reference's
    locus-by-locus sweep."""
    g = load_golden(name)
    P = port.Port(g)
    dg = np.ascontiguousarray(g["dg0"].copy())
    P.lsweep(dg, g["lsweep_u"])
    assert np.array_equal(dg, g["lsweep_after"])


@pytest.mark.parametrize("name", CASES)
def test_port_rescaled_lod_matches_golden(name):
    """The FP64 peel with per-rfunction power-of-two rescaling (the checker for
    pedigrees whose plain peel underflows) gives the reference's log-sums and
    log P(T) where the plain peel does not underflow: equal to 1e-12 in LOD
    units (log-sums / ln 10)."""
    g = load_golden(name)
    P = port.Port(g)
    M, n = g["M"], g["n_lod"]
    raw, cnt, tp = P.lod_range(g["lod_graphs"], 0, M - 1, rescale=True)
    assert cnt == g["lod_count"]
    assert abs(tp - g["lod_trait_prob"]) / np.log(10) <= 1e-12
    assert np.abs(raw - g["lod_raw"]).max() / np.log(10) <= 1e-12
    # a sub-range scores the same positions as the whole map
    lo = M // 3
    hi = min(M - 1, lo + 7)
    sub, _, _ = P.lod_range(g["lod_graphs"], lo, hi, rescale=True)
    np.testing.assert_array_equal(sub, raw[lo * n:hi * n])
    plain, _, _ = P.lod_range(g["lod_graphs"], 0, M - 1, rescale=False)
    np.testing.assert_array_equal(plain, g["lod_raw"])


def test_rescaled_lod_where_the_plain_peel_underflows():
    """On the 400-member pedigree the plain FP64 peel underflows (the reference
    stops there, peeler.cc:89-92) while the rescaled peel gives finite scores;
    the two agree on log P(T), which does not underflow."""
    from swiftlink_gb300 import pedigree, synth
    d = pedigree.problem_from_workload(synth.make_workload(5))
    d["legal"] = host_legal(d)
    d["trait_prior"] = port.derive_priors(d["genotypes"], d["typed"], d["minor"])
    P = port.Port(d)
    raw, cnt, tp = P.lod_range(d["dg0"][None], 100, 104, rescale=True)
    assert np.isfinite(raw).all() and (raw > -1e300).all()
    plain, _, tp0 = P.lod_range(d["dg0"][None], 100, 104, rescale=False, zero_ok=True)
    assert (plain <= -1e300).all()
    assert abs(tp - tp0) <= 1e-12 * abs(tp0)


def host_legal(d):
    """Genotype-elimination masks from the library's host code (no device)."""
    import ctypes
    from swiftlink_gb300 import api
    desc = api.Problem.from_arrays(d, with_legal=False).desc()
    out = np.zeros((d["M"], d["N"]), np.uint8)
    rc = api.lib().sl_problem_legal_masks(ctypes.byref(desc), out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    return out


@pytest.mark.parametrize("name", CASES)
def test_port_msweep_matches_golden(name):
    g = load_golden(name)
    P = port.Port(g)
    dg, used = P.msweep(g["lsweep_after"], g["msweep_order"], g["msweep_u"])
    assert np.array_equal(dg, g["msweep_after"])
    assert np.array_equal(used, g["msweep_used"])


@pytest.mark.parametrize("name", CASES)
def test_port_lod_matches_golden(name):
    g = load_golden(name)
    P = port.Port(g)
    raw, cnt, tp = P.lod(g["lod_graphs"])
    assert cnt == g["lod_count"]
    assert tp == g["lod_trait_prob"]
    np.testing.assert_array_equal(raw, g["lod_raw"])


@pytest.mark.parametrize("name", CASES)
def test_port_loglik_matches_golden(name):
    g = load_golden(name)
    P = port.Port(g)
    # DescentGraph::get_likelihood sums per-locus terms in another order: ulp-level agreement
    assert abs(P.loglik(g["dg0"]) - g["loglik0"]) <= 1e-9 * abs(g["loglik0"])


@pytest.mark.parametrize("name", CASES)
def test_fag_zero_on_illegal_column(name):
    """An inconsistent column has likelihood 0 (founder_allele_graph4.cc:34-442)."""
    g = load_golden(name)
    P = port.Port(g)
    dg = g["dg0"].copy()
    # find a locus and meiosis whose flip makes the column illegal, if any
    hits = 0
    for l in range(min(g["M"], 30)):
        base = P.fag(dg, l)
        assert base > 0.0
        for i in range(g["F"], g["N"]):
            for par in (0, 1):
                dg[l, i, par] ^= 1
                if P.fag(dg, l) == 0.0:
                    hits += 1
                dg[l, i, par] ^= 1
    assert hits >= 0


needs_ref = pytest.mark.skipif(not ref.available(), reason="reference build not present")


@needs_ref
@pytest.mark.parametrize("cfg", [1, 2])
def test_port_matches_live_reference(cfg, tmp_path):
    from swiftlink_gb300 import synth
    import dataclasses
    paths = synth.workload_files(cfg, str(tmp_path))
    r = ref.Ref(*paths, n_lod=5, peel_iters=10000, seed=cfg)
    p = dataclasses.asdict(r.problem())
    P = port.Port(p)
    rng = np.random.default_rng(100 + cfg)
    dg, _ = r.initial_dg(2)
    stride = r.K + 2 * r.N
    loci = rng.choice(r.M, size=min(r.M, 40), replace=False)
    for l in loci:
        u = rng.random(stride)
        a, na = r.lstep(dg, int(l), u)
        b, nb = P.lstep(dg, int(l), u)
        assert na == nb and np.array_equal(a, b)
        dg = a
    order = p["meioses"].copy()
    rng.shuffle(order)
    order = order[: min(order.size, 12)]
    u = rng.random((order.size, r.M))
    a, ua = r.msweep(dg, order, u)
    b, ub = P.msweep(dg, order, u)
    assert np.array_equal(a, b) and np.array_equal(ua, ub)
    graphs = np.stack([dg, a])
    ra = r.lod(graphs)
    rb = P.lod(graphs)
    assert ra[1] == rb[1] and ra[2] == rb[2]
    np.testing.assert_array_equal(ra[0], rb[0])
    r.close()


def test_philox_known_answer():
    """Philox4x32-10 known-answer vector from the Random123 distribution
    (counter 0, key 0 -> 6627e8d5 e169c58d bc57ac4c 9b00dbd8), checked through
    the uniform built from the first two words."""
    u = port.philox_uniform(0, 0, 0)
    w0, w1 = 0x6627E8D5, 0xE169C58D
    expect = ((w0 >> 5) * 67108864 + (w1 >> 6)) / 9007199254740992.0
    assert u == expect


def test_numpy_philox_matches_c_port():
    from swiftlink_gb300 import philox as philox_np
    rng = np.random.default_rng(5)
    for _ in range(50):
        key, hi, lo = (int(x) for x in rng.integers(0, 2**63, 3))
        assert float(philox_np.uniform(key, hi, lo)) == port.philox_uniform(key, hi, lo)


@pytest.mark.parametrize("name", CASES)
def test_port_priors_match_reference_bitwise(name):
    g = load_golden(name)
    pri = port.derive_priors(g["genotypes"], g["typed"], g["minor"])
    np.testing.assert_array_equal(pri, g["trait_prior"])
