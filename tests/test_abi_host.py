"""CPU checks of the C-ABI library: it loads, exports every symbol the public
header declares, and its host-side tables (genotype elimination, L-sampler
priors, log P(T)) equal the reference's on the golden cases.  No kernels run."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, CASES, load_golden
from swiftlink_gb300 import api


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()


def header_symbols():
    src = open(os.path.join(ROOT, "include", "swiftlink_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sl_[a-z_0-9]+)\s*\(", src)))


def test_exports_every_declared_symbol():
    L = api.lib()
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(api.EXPORTED) <= set(syms)


def test_python_constants_match_the_header():
    """Every SL_* integer constant the Python mirror defines has the header's value."""
    src = open(os.path.join(ROOT, "include", "swiftlink_gb300.h")).read()
    defs = {k: int(v) for k, v in re.findall(r"#define\s+(SL_[A-Z0-9_]+)\s+(-?\d+)\b", src)}
    mirrored = {k: getattr(api, k) for k in dir(api) if k.startswith("SL_") and isinstance(getattr(api, k), int)}
    assert len(mirrored) >= 15
    for k, v in mirrored.items():
        assert k in defs, k
        assert defs[k] == v, (k, defs[k], v)


def test_version_and_null_handling():
    L = api.lib()
    assert b"sm_103a" in L.sl_version()
    assert L.sl_create(None, None, None) == api.SL_EINVAL
    assert len(L.sl_last_error(None)) > 0


@pytest.mark.parametrize("name", CASES)
def test_legal_masks_match_reference(name):
    g = load_golden(name)
    prob = api.Problem.from_arrays(g, with_legal=False)
    desc = prob.desc()
    out = np.zeros((g["M"], g["N"]), np.uint8)
    rc = api.lib().sl_problem_legal_masks(ctypes.byref(desc), out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    np.testing.assert_array_equal(out, g["legal"])


@pytest.mark.parametrize("name", CASES)
def test_trait_priors_match_reference_bitwise(name):
    g = load_golden(name)
    prob = api.Problem.from_arrays(g)
    desc = prob.desc()
    out = np.zeros((g["M"], g["N"], 4))
    rc = api.lib().sl_problem_trait_priors(ctypes.byref(desc), out.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    np.testing.assert_array_equal(out, g["trait_prior"])


@pytest.mark.parametrize("name", CASES)
def test_trait_prob_matches_reference(name):
    g = load_golden(name)
    prob = api.Problem.from_arrays(g)
    desc = prob.desc()
    tp = ctypes.c_double()
    rc = api.lib().sl_problem_trait_prob(ctypes.byref(desc), ctypes.byref(tp))
    assert rc == 0
    assert abs(tp.value - g["lod_trait_prob"]) <= 1e-12 * max(1.0, abs(g["lod_trait_prob"]))


def test_inconsistent_genotypes_are_rejected():
    g = load_golden("loop")
    geno = g["genotypes"].copy()
    # child homozygous B with a homozygous-A parent: a Mendelian impossibility
    child = next(i for i in range(g["N"]) if g["mother"][i] >= 0)
    geno[0, child] = 3
    geno[0, g["mother"][child]] = 2
    d = dict(g, genotypes=geno, typed=np.ones(g["N"], np.uint8))
    prob = api.Problem.from_arrays(d, with_legal=False)
    desc = prob.desc()
    out = np.zeros((g["M"], g["N"]), np.uint8)
    rc = api.lib().sl_problem_legal_masks(ctypes.byref(desc), out.ctypes.data_as(ctypes.c_void_p))
    assert rc == api.SL_EINVAL
    assert b"inconsistent" in api.lib().sl_last_error(None)


def test_create_without_gpu_fails_cleanly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    g = load_golden("loop")
    with pytest.raises(api.SwiftLinkError) as e:
        api.Context(api.Problem.from_arrays(g))
    assert e.value.code == api.SL_ENODEV


@pytest.mark.parametrize("name", CASES)
def test_compiled_lod_program_matches_reference(name):
    """The host compiler of the batched trait peel, evaluated in FP64, gives the
    reference's per-position log-likelihood ratios."""
    g = load_golden(name)
    prob = api.Problem.from_arrays(g)
    desc = prob.desc()
    dg = np.ascontiguousarray(g["lod_graphs"][0], np.int32)
    n = g["n_lod"]
    raw_one = None
    from oracle import port
    raw_one, _, _ = port.Port(g).lod(dg[None])
    rng = np.random.default_rng(3)
    loci = sorted(set([0, g["M"] - 2] + list(rng.integers(0, g["M"] - 1, 12))))
    fn = api.lib().sl_problem_lod_program_eval
    for l in loci:
        for o in range(n):
            v = ctypes.c_double()
            rc = fn(ctypes.byref(desc), dg.ctypes.data_as(ctypes.c_void_p), int(l), o, ctypes.byref(v))
            assert rc == 0
            assert abs(v.value - raw_one[l * n + o]) <= 1e-9 * max(1.0, abs(raw_one[l * n + o])), (l, o)


@pytest.mark.parametrize("name", CASES)
def test_disease_probs_restatement_matches_reference(name):
    from swiftlink_gb300.workloads import disease_probs
    g = load_golden(name)
    dp = disease_probs(g["affection"], g["mother"] < 0, g["freq"], g["penetrance"])
    np.testing.assert_array_equal(dp, g["disease_prob"])
