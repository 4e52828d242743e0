"""The swift_gb300 program: LINKAGE files in, the LOD table out.

CPU: the problem tables it builds from the files (its --dumpproblem mode)
against the reference's own tables for the same files (the golden cfg1 and
cfg2 problems, which the reference's parsers built from these synthetic
files: member order, parents, genotypes, disease probabilities, theta,
partial theta, MAFs, positions), families of one pedigree file kept apart,
and the input errors it reports.  GPU: the LOD table it writes against the
library driven through the Python API with the same problem, seeds and run
options, with and without MC3 (one context of tempered chains per run, the
runs' tables merged as LODscores::merge_results does); the CODA trace lines
(MarkovChain::run, markov_chain.cc:357-370); a traced run's table is the
untraced run's table, also when MC3 exchanges fall inside traced spans.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from swiftlink_gb300 import api, cli, synth


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()


def run_cli(*args, check=True):
    r = subprocess.run([cli.path(), *[str(a) for a in args]], capture_output=True, text=True, timeout=600)
    if check and r.returncode != 0:
        raise AssertionError(f"swift_gb300 exited {r.returncode}\n{r.stdout}\n{r.stderr}")
    return r


def dump(tmp_path, ped, mapf, dat, *extra):
    out = tmp_path / "problem.txt"
    run_cli("-p", ped, "-m", mapf, "-d", dat, "-D", out, *extra)
    return cli.read_dump(str(out))


def golden_problem(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz" if name == "cfg1" else f"{name}_problem.npz"))
    return {k: z[k] for k in z.files}


def test_table_writer_matches_the_reference_writer(tmp_path):
    """The LOD table file for given log-sums, count and log P(T) (the
    program's -W mode) is byte-identical to the reference's
    LinkageWriter::write (linkage_writer.cc:14-89) on the same values and the
    same LINKAGE files (positions from the map, names, number formatting)."""
    from oracle import ref
    if not ref.available():
        pytest.skip("the reference build exists only where the reference sources are")
    ped, mapf, dat = synth.workload_files(1, str(tmp_path))
    r = ref.Ref(ped, mapf, dat, n_lod=5, peel_iters=100, seed=3)
    npos = (r.M - 1) * r.n_lod
    rng = np.random.default_rng(5)
    raw = -800.0 + 30.0 * rng.standard_normal(npos)
    count, tp = 123, -411.25
    r.write_table(raw, count, tp, str(tmp_path / "ref.lod"))
    r.close()
    src = tmp_path / "logsums.txt"
    src.write_text(f"{count} {tp!r}\n" + "\n".join(repr(float(x)) for x in raw) + "\n")
    run_cli("-p", ped, "-m", mapf, "-d", dat, "-W", src, "-o", tmp_path / "ours.lod")
    assert (tmp_path / "ours.lod").read_bytes() == (tmp_path / "ref.lod").read_bytes()


@pytest.mark.parametrize("cfg", [1, 2])
def test_tables_match_the_reference_parse(tmp_path, cfg):
    files = synth.workload_files(cfg, str(tmp_path))
    (d,) = dump(tmp_path, *files)
    g = golden_problem(f"cfg{cfg}")
    assert (d["N"], d["F"], d["M"]) == (int(g["N"]), int(g["F"]), int(g["M"]))
    for k in ("mother", "father", "sex", "affection", "typed", "genotypes"):
        np.testing.assert_array_equal(d[k], g[k], err_msg=k)
    for k in ("disease_prob", "theta", "partial", "minor", "gpos"):
        np.testing.assert_allclose(d[k], g[k], rtol=1e-14, atol=0, err_msg=k)
    assert d["model"][0] == pytest.approx(float(g["freq"]), rel=1e-12)
    np.testing.assert_array_equal(d["model"][1:], g["penetrance"])
    # the peel sequence is the library's own for the same members
    ot, op = api.peel_sequence(d["mother"].astype(np.int32), d["father"].astype(np.int32))[:2]
    np.testing.assert_array_equal(d["op_type"], ot)
    np.testing.assert_array_equal(d["op_peel"], op)


def two_family_files(tmp_path):
    w1 = synth.make_workload(1)
    w2 = synth.make_workload(1, seed=4242)
    w2.famid = "fam2"
    ped, mapf, dat = synth.write_linkage(w1, str(tmp_path / "two"))
    p2 = synth.write_linkage(w2, str(tmp_path / "second"))[0]
    with open(ped, "a") as f, open(p2) as g:
        f.write(g.read())
    one = [synth.write_linkage(w, str(tmp_path / f"only{k}")) for k, w in enumerate((w1, w2))]
    return (ped, mapf, dat), one


def test_families_are_kept_apart(tmp_path):
    both, one = two_family_files(tmp_path)
    fams = dump(tmp_path, *both)
    assert [f["id"] for f in fams] == ["1", "fam2"]
    for k, f in enumerate(fams):
        (single,) = dump(tmp_path, one[k][0], both[1], both[2])
        for key in ("ids", "mother", "father", "genotypes", "disease_prob", "op_peel"):
            np.testing.assert_array_equal(np.asarray(f[key]), np.asarray(single[key]), err_msg=key)


def test_affected_only_makes_the_others_unknown(tmp_path):
    files = synth.workload_files(1, str(tmp_path))
    (d,) = dump(tmp_path, *files)
    (a,) = dump(tmp_path, *files, "-a")
    np.testing.assert_array_equal(a["affection"], np.where(d["affection"] == 2, 2, 0))
    unk = a["affection"] == 0
    nonf = d["mother"] >= 0
    np.testing.assert_array_equal(a["disease_prob"][unk & nonf], 0.25)


def _write(path, text):
    path.write_text(text)
    return str(path)


def test_input_errors_are_reported(tmp_path):
    files = synth.workload_files(1, str(tmp_path))
    ped, mapf, dat = files
    lines = open(ped).read().splitlines()
    # a third allele
    t = lines[3].split()
    t[6] = "3"
    bad = _write(tmp_path / "bad_allele.ped", "\n".join(lines[:3] + [" ".join(t)] + lines[4:]) + "\n")
    r = run_cli("-p", bad, "-m", mapf, "-d", dat, "-D", tmp_path / "x", check=False)
    assert r.returncode == 1 and "genotype" in r.stderr
    # bad sex code
    t = lines[3].split()
    t[4] = "7"
    bad = _write(tmp_path / "bad_sex.ped", "\n".join(lines[:3] + [" ".join(t)] + lines[4:]) + "\n")
    r = run_cli("-p", bad, "-m", mapf, "-d", dat, "-D", tmp_path / "x", check=False)
    assert r.returncode == 1 and "sex" in r.stderr
    # a parent that is not in the family
    t = lines[-1].split()
    t[2] = "999"
    bad = _write(tmp_path / "bad_parent.ped", "\n".join(lines[:-1] + [" ".join(t)]) + "\n")
    r = run_cli("-p", bad, "-m", mapf, "-d", dat, "-D", tmp_path / "x", check=False)
    assert r.returncode == 1 and "parent" in r.stderr
    # fewer markers in the map than in the dat file
    mlines = open(mapf).read().splitlines()
    short = _write(tmp_path / "short.map", "\n".join(mlines[:-1]) + "\n")
    r = run_cli("-p", ped, "-m", short, "-d", dat, "-D", tmp_path / "x", check=False)
    assert r.returncode == 1 and "markers" in r.stderr
    # sex-linked analysis is refused, as the reference's GPU path refuses it
    dl = open(dat).read().splitlines()
    h = dl[0].split()
    h[2] = "1"
    xdat = _write(tmp_path / "x.dat", "\n".join([" ".join(h)] + dl[1:]) + "\n")
    r = run_cli("-p", ped, "-m", mapf, "-d", xdat, "-D", tmp_path / "x", check=False)
    assert r.returncode == 1 and "sex-linked" in r.stderr
    # option values
    r = run_cli("-p", ped, "-m", mapf, "-d", dat, "-i", "abc", check=False)
    assert r.returncode == 1 and "-i" in r.stderr
    r = run_cli("-p", ped, "-m", mapf, "-d", dat, "-l", "1.5", check=False)
    assert r.returncode == 1
    r = run_cli("-h", check=False)
    assert r.returncode == 0 and "Usage" in r.stderr


# ---------------------------------------------------------------------------
# GPU: the program end to end
# ---------------------------------------------------------------------------

def api_lod_tables(fams, runs, si, iterations, burnin, period, lprob, seed, exact):
    """What the program computes, driven through the Python API."""
    prec = dict(lod_precision=api.SL_LOD_FP64 if exact else api.SL_LOD_FP32_RESCALED,
                sampler_precision=api.SL_SAMPLER_EXACT if exact else api.SL_SAMPLER_FAST,
                lod_flags=api.SL_LOD_ZERO_OK)
    ctxs = []
    for f, d in enumerate(fams):
        ot, op, cut, prev, ch = api.peel_sequence(d["mother"].astype(np.int32), d["father"].astype(np.int32))
        arrays = dict(N=d["N"], F=d["F"], M=d["M"], n_lod=5, mother=d["mother"].astype(np.int32),
                      father=d["father"].astype(np.int32), sex=d["sex"].astype(np.int32),
                      typed=d["typed"].astype(np.uint8), genotypes=d["genotypes"].astype(np.uint8),
                      disease_prob=d["disease_prob"], theta=d["theta"], partial=d["partial"], minor=d["minor"],
                      op_type=ot, op_peel=op, op_cutset=cut, op_prev=prev, op_children=ch)
        ctx = api.Context(api.Problem.from_arrays(arrays, with_legal=False), n_chains=runs, **prec)
        ctx.sequential_imputation_run(si, seed + f)
        ctxs.append(ctx)
    b = api.Batch(ctxs)
    b.run(iterations=iterations, burnin=burnin, period=period, lprob=lprob, seed=seed)
    out = [api.lod_table(*c.lod_results()) for c in ctxs]
    b.close()
    for c in ctxs:
        c.close()
    return out


def positions(d, n=5):
    g = d["gpos"]
    inv = lambda r: -0.5 * np.log(1 - 2 * r)   # noqa: E731
    return np.array([100 * (g[i] + inv(d["partial"][i] * (j + 1))) for i in range(d["M"] - 1) for j in range(n)])


def check_table(t, fams, lods, tol):
    d0 = fams[0]
    assert [m[0] for m in t["markers"]] == [f"snp{j + 1}" for j in range(d0["M"])]
    np.testing.assert_allclose([m[1] for m in t["markers"]], 100 * d0["gpos"], rtol=1e-5)
    np.testing.assert_allclose(t["position"], positions(d0), rtol=1e-5)
    total = np.sum(lods, axis=0)
    assert np.all(np.isfinite(t["lod"]))
    np.testing.assert_allclose(t["lod"], total, rtol=1e-5, atol=tol)
    if len(fams) > 1:
        np.testing.assert_allclose(t["per_family"], np.stack(lods, axis=1), rtol=1e-5, atol=tol)
    else:
        assert t["per_family"].size == 0 or t["per_family"].shape[1] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [True, False])
def test_lod_table_matches_the_library(tmp_path, exact):
    both, _ = two_family_files(tmp_path)
    fams = dump(tmp_path, *both)
    seedf = _write(tmp_path / "seeds", "77\n")
    opts = dict(runs=2, si=20, iterations=300, burnin=100, period=10, lprob=0.5, seed=77)
    out = tmp_path / "lod.out"
    args = ["-p", both[0], "-m", both[1], "-d", both[2], "-o", out, "-R", opts["runs"], "-s", opts["si"],
            "-i", opts["iterations"], "-b", opts["burnin"], "-x", opts["period"], "-l", opts["lprob"], "-r", seedf]
    run_cli(*args, *(["-E"] if exact else []))
    t = cli.read_lod_table(str(out))
    lods = api_lod_tables(fams, exact=exact, **opts)
    # exact: the same FP64 arithmetic, equal to the 6 printed digits; fast: the
    # batched scorer may pick another kernel, each within 1e-3 of FP64
    check_table(t, fams, lods, 2e-6 if exact else 1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("mc3", [False, True])
def test_trace_lines_and_the_table_do_not_depend_on_tracing(tmp_path, mc3):
    ped, mapf, dat = synth.workload_files(1, str(tmp_path))
    seedf = _write(tmp_path / "seeds", "5\n")
    common = ["-p", ped, "-m", mapf, "-d", dat, "-R", 2, "-s", 10, "-i", 45, "-b", 20, "-x", 10, "-r", seedf, "-E"]
    if mc3:   # exchanges every 7 iterations: not aligned with the traced spans
        common += ["-M", "-z", 3, "-y", 7]
    run_cli(*common, "-o", tmp_path / "plain.out")
    run_cli(*common, "-o", tmp_path / "traced.out", "-T", "-P", tmp_path / "tr")
    assert (tmp_path / "plain.out").read_text() == (tmp_path / "traced.out").read_text()
    for r in range(2):
        lines = (tmp_path / f"tr.ped1.run{r}").read_text().splitlines()
        assert lines[0] == "iteration likelihood"
        its = [int(x.split("\t")[0]) for x in lines[1:]]
        # scoring iterations i >= 20, i % 10 == 0 of i < 65, written as i + 1
        assert its == [21, 31, 41, 51, 61]
        ll = np.array([float(x.split("\t")[1]) for x in lines[1:]])
        assert np.all(np.isfinite(ll)) and np.all(ll < 0)


def log_sum(a, b):
    """log_sum (logarithms.cc:14-25) elementwise, LOG_ZERO = -DBL_MAX."""
    lz = -np.finfo(np.float64).max
    return np.where(a == lz, b, np.where(b == lz, a, np.log(np.exp(b - a) + 1) + a))


@pytest.mark.gpu
def test_mc3_runs_match_the_library(tmp_path):
    ped, mapf, dat = synth.workload_files(1, str(tmp_path))
    (d,) = dump(tmp_path, ped, mapf, dat)
    seed, R, Z, Y = 31, 2, 3, 5
    seedf = _write(tmp_path / "seeds", f"{seed}\n")
    out = tmp_path / "mc3.out"
    run_cli("-p", ped, "-m", mapf, "-d", dat, "-o", out, "-R", R, "-s", 10, "-i", 200, "-b", 50, "-x", 10,
            "-r", seedf, "-E", "-M", "-z", Z, "-y", Y, "-v")
    t = cli.read_lod_table(str(out))
    temps = [1.0] + [1.0 / (1.0 + 0.001 * 2.0 ** i) for i in range(1, Z)]
    ot, op, cut, prev, ch = api.peel_sequence(d["mother"].astype(np.int32), d["father"].astype(np.int32))
    arrays = dict(N=d["N"], F=d["F"], M=d["M"], n_lod=5, mother=d["mother"].astype(np.int32),
                  father=d["father"].astype(np.int32), sex=d["sex"].astype(np.int32),
                  typed=d["typed"].astype(np.uint8), genotypes=d["genotypes"].astype(np.uint8),
                  disease_prob=d["disease_prob"], theta=d["theta"], partial=d["partial"], minor=d["minor"],
                  op_type=ot, op_peel=op, op_cutset=cut, op_prev=prev, op_children=ch)
    ctxs = []
    for r in range(R):
        c = api.Context(api.Problem.from_arrays(arrays, with_legal=False), n_chains=Z,
                        lod_precision=api.SL_LOD_FP64, sampler_precision=api.SL_SAMPLER_EXACT,
                        lod_flags=api.SL_LOD_ZERO_OK)
        c.set_temperatures(temps)
        c.sequential_imputation_run(10, seed + r)
        ctxs.append(c)
    b = api.Batch(ctxs)
    b.run(iterations=200, burnin=50, period=10, lprob=0.5, seed=seed, exchange_period=Y)
    res = [c.lod_results() for c in ctxs]
    stats = [c.mc3_stats() for c in ctxs]
    b.close()
    for c in ctxs:
        c.close()
    raw = log_sum(res[0][0], res[1][0])
    lod = api.lod_table(raw, res[0][1] + res[1][1], res[0][2])
    check_table(t, [d], [lod], 2e-6)
    # one exchange proposed per full spurt of Y iterations in each run
    assert all(int(p.sum()) == 250 // Y for _, p in stats)


@pytest.mark.gpu
def test_long_runs_compile_the_lsampler_with_the_same_table(tmp_path):
    """With -J, runs of 10,000 iterations or more use the L-sampler compiled
    for the pedigree; it draws the generic kernel's graphs bit for bit, so the
    table equals the one of the same run with -G (generic kernel)."""
    ped, mapf, dat = synth.workload_files(1, str(tmp_path))
    seedf = _write(tmp_path / "seeds", "3\n")
    common = ["-p", ped, "-m", mapf, "-d", dat, "-R", 2, "-s", 10, "-i", 6000, "-b", 4000, "-x", 50, "-r", seedf]
    run_cli(*common, "-o", tmp_path / "spec.out", "-J")
    run_cli(*common, "-o", tmp_path / "gen.out", "-G")
    assert (tmp_path / "spec.out").read_text() == (tmp_path / "gen.out").read_text()
