"""The trait-peel adjoint specialised to one pedigree (sl_adjjit.cc), on the host.

sl_problem_adjoint_source writes out the CUDA C++ source of the specialised
adjoint for a problem.  Here that source is compiled as plain host C++
(tests/cuda_host_prelude.h defines the CUDA qualifiers and builtins it uses),
its kernel run for every thread of one block on the CPU, and its gradients
checked against the FP64 host adjoint (sl_problem_trait_backward_eval, itself
checked against finite differences in test_trait_adjoint.py) within the
same 1e-4 of each component's norm.  This tests the generator's peel, its
reverse and its arena layout without a GPU; the same source is compiled with
NVRTC for sm_103a, and the device runs are in test_trait_adjoint.py.
"""
import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import CASES, load_golden
from swiftlink_gb300 import api
from swiftlink_gb300.workloads import disease_probs

HERE = os.path.dirname(os.path.abspath(__file__))
GRAD_RTOL = 1e-4
DOMINANT = ((0.01, 0.8, 0.9), 1e-3)
THREADS = 128


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()


def with_model(g, pen, freq):
    d = dict(g)
    d["penetrance"] = np.array(pen, np.float64)
    d["freq"] = np.float64(freq)
    d["disease_prob"] = disease_probs(g["affection"], g["mother"] < 0, freq, pen)
    return d


def source(desc, compile_=False, variant=0):
    f = api.lib().sl_problem_adjoint_source
    n = ctypes.c_int64()
    shapes = ctypes.c_int32()
    ms = ctypes.c_double()
    assert f(ctypes.byref(desc), variant, 0, None, 0, ctypes.byref(n), ctypes.byref(shapes), None) == 0
    buf = ctypes.create_string_buffer(n.value + 1)
    rc = f(ctypes.byref(desc), variant, int(compile_), buf, n.value + 1, None, None, ctypes.byref(ms))
    assert rc == 0, api.lib().sl_last_error(None)
    return buf.value.decode(), shapes.value, ms.value


def disease_grad(d):
    """d disease_prob[person][state] / d (pen HOMO_U, HETERO, HOMO_A, freq)
    (person.cc:85-119, disease_model.cc:139-187), as the device table."""
    pen, q = d["penetrance"], float(d["freq"])
    unph = [0, 2, 1, 1]
    prior = [(1 - q) ** 2, q * (1 - q), q * q]
    dprior = [-2 * (1 - q), 1 - 2 * q, 2 * q]
    out = np.zeros((len(d["mother"]), 4, 4), np.float32)
    for p, a in enumerate(d["affection"]):
        for s in range(4):
            t = unph[s]
            if d["mother"][p] < 0:
                if a == 2:
                    out[p, s, t], out[p, s, 3] = prior[t], dprior[t] * pen[t]
                elif a == 1:
                    out[p, s, t], out[p, s, 3] = -prior[t], dprior[t] * (1 - pen[t])
                else:
                    out[p, s, 3] = dprior[t]
            elif a == 2:
                out[p, s, t] = 1.0
            elif a == 1:
                out[p, s, t] = -1.0
    return out


def pack(graphs, N, F, M):
    W = (2 * (N - F) + 31) // 32
    n = graphs.shape[0]
    bits = graphs[:, :, F:, :].reshape(n, M, 2 * (N - F)).astype(np.uint64)
    out = np.zeros((n, M, W), np.uint64)
    for b in range(2 * (N - F)):
        out[:, :, b >> 5] |= bits[:, :, b] << np.uint64(b & 31)
    return out.astype(np.uint32)


DRIVER = r'''
extern "C" void host_run(unsigned blocks, const u32* graphs, long long gw, long long task0, long long ntask,
                         double* grad, int* status, const float* partial, float* arena, const float* dprob,
                         const float4* dgrad, int zero_ok) {
    gridDim.x = blocks;
    for (unsigned b = 0; b < blocks; ++b)
        for (unsigned t = 0; t < %d; ++t) {
            blockIdx.x = b;
            threadIdx.x = t;
            sl_adj_jit(graphs, gw, task0, ntask, grad, status, partial, arena, dprob, dgrad, zero_ok);
        }
}
''' % THREADS


def host_kernel(src, tmp_path, tag):
    path = os.path.join(tmp_path, f"adj_{tag}.cc")
    so = os.path.join(tmp_path, f"adj_{tag}.so")
    with open(path, "w") as f:
        f.write('#include "cuda_host_prelude.h"\n' + src + DRIVER)
    subprocess.run(["g++", "-O1", "-shared", "-fPIC", "-I", HERE, "-o", so, path], check=True)
    return ctypes.CDLL(so)


def run_host(d, graph, ntask, tmp_path, tag):
    """The generated kernel of problem d over the first ntask positions of
    graph, run on the host; returns its gradients [ntask][6]."""
    prob = api.Problem.from_arrays(d)
    desc = prob.desc()
    src, shapes, _ = source(desc)
    assert shapes >= 1
    lib = host_kernel(src, str(tmp_path), tag)
    half = int(re.search(r"#define HB (\d+)", src).group(1)) // THREADS
    N, F, M, K = int(d["N"]), int(d["F"]), int(d["M"]), len(d["op_cutset"])
    pk = np.ascontiguousarray(pack(graph[None], N, F, M))
    blocks = 2
    grad = np.zeros((ntask, 6))
    status = np.zeros(1, np.int32)
    partial = np.asarray(d["partial"], np.float32)
    dprob = np.ascontiguousarray(d["disease_prob"], np.float32)
    dgrad = disease_grad(d)
    arena = np.zeros(blocks * (2 * half + K) * THREADS, np.float32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    run = lib.host_run
    run.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_longlong,
                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                    ctypes.c_void_p, ctypes.c_int]
    run(blocks, P(pk), pk.shape[1] * pk.shape[2], 0, ntask, P(grad), P(status), P(partial), P(arena), P(dprob),
        P(dgrad), 0)
    assert status[0] == 0
    return grad


def host_fp64(d, graph, ntask):
    desc = api.Problem.from_arrays(d).desc()
    n = int(d["n_lod"])
    want = np.zeros((ntask, 6))
    hb = api.lib().sl_problem_trait_backward_eval
    for u in range(ntask):
        l, o = divmod(u, n)
        assert hb(ctypes.byref(desc), graph.ctypes.data_as(ctypes.c_void_p), l, o,
                  want[u].ctypes.data_as(ctypes.c_void_p)) == 0
    return want


def assert_close(grad, want):
    for k in range(6):
        err = np.linalg.norm(grad[:, k] - want[:, k]) / max(np.linalg.norm(want[:, k]), 1e-300)
        assert err <= GRAD_RTOL, (k, err)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
@pytest.mark.parametrize("model", ["recessive", "dominant"])
@pytest.mark.parametrize("name", CASES)
def test_generated_adjoint_matches_host_fp64(name, model, tmp_path):
    """Every position of the first golden graph, two blocks of threads (so
    each thread's arena column holds several tasks one after another)."""
    g = load_golden(name)
    d = g if model == "recessive" else with_model(g, *DOMINANT)
    graph = np.ascontiguousarray(g["lod_graphs"][0], np.int32)
    ntask = (int(g["M"]) - 1) * int(g["n_lod"])
    assert_close(run_host(d, graph, ntask, tmp_path, f"{name}_{model}"), host_fp64(d, graph, ntask))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
def test_generated_adjoint_large_pedigree_matches_host_fp64(tmp_path):
    """The 120-member, 2000-SNP pedigree under the dominant model (27
    operation shapes, cutsets of up to four members, parent peels with
    several children): its starting graph's first 60 positions."""
    from swiftlink_gb300.workloads import load_problem
    g = load_problem("cfg2")
    d = with_model(g, *DOMINANT)
    graph = np.ascontiguousarray(g["dg0"], np.int32)
    assert_close(run_host(d, graph, 60, tmp_path, "cfg2"), host_fp64(d, graph, 60))


@pytest.mark.parametrize("variant", range(api.SL_ADJOINT_VARIANTS))
def test_generated_adjoint_compiles_for_sm103a(variant):
    """The same source through NVRTC for sm_103a (no device needed), at each
    register budget the library compiles."""
    g = load_golden("cfg1")
    src, shapes, ms = source(api.Problem.from_arrays(with_model(g, *DOMINANT)).desc(), compile_=True,
                             variant=variant)
    assert shapes >= 1 and ms > 0
    assert "__launch_bounds__(128, %d)" % (4, 8)[variant] in src
