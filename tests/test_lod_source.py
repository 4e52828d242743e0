"""The batched LOD scorer specialised to a problem (sl_jit.cc), on the host.

sl_problem_lod_source writes out the CUDA C++ source of the kernel that an
SL_LOD_FP32_RESCALED context compiles with NVRTC: the problem's trait peel as
straight-line FP32 code with per-rfunction power-of-two rescaling, then the
log-likelihood ratio of every (graph, interval, position) in FP64.  Here the
register form of that source is compiled as plain host C++
(tests/cuda_host_prelude.h), its kernel run for every thread of a block on the
CPU, and each graph's per-position values checked against the C restatement's
FP64 peel (oracle/port.py, pinned to the reference) within the FP32 LOD
tolerance of the device tests: |dLOD| <= 1e-3, i.e. 1e-3 ln 10 in the natural
log-likelihood ratio.
"""
import ctypes
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import CASES, load_golden
from swiftlink_gb300 import api

HERE = os.path.dirname(os.path.abspath(__file__))
THREADS = 128
TOL = 1e-3 * math.log(10.0)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from swiftlink_gb300 import build
    build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(os.path.dirname(HERE), "oracle"), "port"], check=True)


def pack(graphs, N, F, M):
    W = (2 * (N - F) + 31) // 32
    n = graphs.shape[0]
    bits = graphs[:, :, F:, :].reshape(n, M, 2 * (N - F)).astype(np.uint64)
    out = np.zeros((n, M, W), np.uint64)
    for b in range(2 * (N - F)):
        out[:, :, b >> 5] |= bits[:, :, b] << np.uint64(b & 31)
    return out.astype(np.uint32)


DRIVER = r'''
extern "C" void host_run(unsigned blocks, const u32* graphs, long long gw, int G, double* vals, int* status,
                         const float* partial, const double* lt, const double* la) {
    gridDim.x = blocks;
    for (unsigned b = 0; b < blocks; ++b)
        for (unsigned t = 0; t < S; ++t) {
            blockIdx.x = b;
            threadIdx.x = t;
            sl_lod_jit(graphs, gw, G, vals, status, partial, lt, la);
        }
}
'''


def lod_source(desc, shared=0, compile_=False):
    f = api.lib().sl_problem_lod_source
    n = ctypes.c_int64()
    assert f(ctypes.byref(desc), shared, THREADS, api.SL_LOD_ZERO_OK, 0, None, 0, ctypes.byref(n), None, None) == 0
    buf = ctypes.create_string_buffer(n.value + 1)
    ms = ctypes.c_double()
    rc = f(ctypes.byref(desc), shared, THREADS, api.SL_LOD_ZERO_OK, int(compile_), buf, n.value + 1, None, None,
           ctypes.byref(ms))
    assert rc == 0, api.lib().sl_last_error(None)
    return buf.value.decode()


def check_against_port(g, graphs, tmp_path):
    """The generated kernel over graphs [G][M][N][2] of problem g, run on the
    host, against the restatement's FP64 peel graph by graph."""
    from oracle import port
    prob = api.Problem.from_arrays(g)
    src = lod_source(prob.desc())
    path, so = os.path.join(tmp_path, "lod.cc"), os.path.join(tmp_path, "lod.so")
    with open(path, "w") as f:
        f.write('#include "cuda_host_prelude.h"\n' + src + DRIVER)
    subprocess.run(["g++", "-O1", "-shared", "-fPIC", "-I", HERE, "-o", so, path], check=True)
    lib = ctypes.CDLL(so)
    N, F, M, n = int(g["N"]), int(g["F"]), int(g["M"]), int(g["n_lod"])
    graphs = np.ascontiguousarray(graphs, np.int32)
    G = graphs.shape[0]
    pk = np.ascontiguousarray(pack(graphs, N, F, M))
    npos = (M - 1) * n
    vals = np.zeros(G * npos)
    status = np.zeros(1, np.int32)
    theta = np.asarray(g["theta"], np.float64)
    partial = np.asarray(g["partial"], np.float32)
    lt, la = np.log(theta), np.log(1.0 - theta)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    run = lib.host_run
    run.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p,
                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    blocks = 2
    run(blocks, P(pk), M * pk.shape[2], G, P(vals), P(status), P(partial), P(lt), P(la))
    assert status[0] == 0
    oracle = port.Port(g)
    for b in range(G):
        want, _, _ = oracle.lod(graphs[b:b + 1])
        got = vals[b * npos:(b + 1) * npos]
        ok = want > -1e300
        assert np.array_equal(ok, got > -1e300)
        err = np.abs(got[ok] - want[ok]).max()
        assert err <= TOL, (b, err)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
@pytest.mark.parametrize("name", CASES)
def test_generated_lod_kernel_matches_the_fp64_peel(name, tmp_path):
    """Every golden graph of the case, every interval and position."""
    g = load_golden(name)
    check_against_port(g, g["lod_graphs"], tmp_path)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
def test_generated_lod_kernel_large_pedigree(tmp_path):
    """The 120-member, 2000-SNP pedigree (3 loops, 35 affected): its starting
    graph at every one of the 9,995 positions."""
    from oracle import port
    from swiftlink_gb300.workloads import load_problem
    g = load_problem("cfg2")
    desc = api.Problem.from_arrays(g, with_legal=False).desc()
    g["legal"] = np.zeros((g["M"], g["N"]), np.uint8)
    assert api.lib().sl_problem_legal_masks(ctypes.byref(desc), g["legal"].ctypes.data_as(ctypes.c_void_p)) == 0
    g["trait_prior"] = port.derive_priors(g["genotypes"], g["typed"], g["minor"])
    check_against_port(g, g["dg0"][None], tmp_path)


@pytest.mark.parametrize("shared", [0, 1])
def test_generated_lod_kernel_compiles_for_sm103a(shared):
    """Both storage forms of the 30-member case through NVRTC for sm_103a (no
    device needed)."""
    g = load_golden("cfg1")
    prob = api.Problem.from_arrays(g)
    src = lod_source(prob.desc(), shared=shared, compile_=True)
    assert "sl_lod_jit" in src and ("extern __shared__" in src) == bool(shared)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
@pytest.mark.parametrize("name", CASES)
def test_generated_lod_kernel_forms_agree(name, tmp_path):
    """The shared-memory form (values in a per-thread column of the block's
    arena, immediate offsets) against the register form on the host: the
    same operations in the same order, so the same values."""
    g = load_golden(name)
    prob = api.Problem.from_arrays(g)
    N, F, M, n = int(g["N"]), int(g["F"]), int(g["M"]), int(g["n_lod"])
    graphs = np.ascontiguousarray(g["lod_graphs"], np.int32)
    G = graphs.shape[0]
    pk = np.ascontiguousarray(pack(graphs, N, F, M))
    npos = (M - 1) * n
    theta = np.asarray(g["theta"], np.float64)
    partial = np.asarray(g["partial"], np.float32)
    lt, la = np.log(theta), np.log(1.0 - theta)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    out = []
    for shared in (0, 1):
        desc = prob.desc()
        slots = ctypes.c_int32()
        f = api.lib().sl_problem_lod_source
        ln = ctypes.c_int64()
        assert f(ctypes.byref(desc), shared, THREADS, api.SL_LOD_ZERO_OK, 0, None, 0, ctypes.byref(ln),
                 ctypes.byref(slots), None) == 0
        src = lod_source(desc, shared=shared)
        # the block's shared arena as a host array: the emulated threads run one after another
        arena = "" if not shared else "float sh[%d];\n" % (THREADS * max(1, slots.value))
        path, so = os.path.join(tmp_path, f"lod{shared}.cc"), os.path.join(tmp_path, f"lod{shared}.so")
        with open(path, "w") as fh:
            fh.write('#include "cuda_host_prelude.h"\n' + arena + src.replace("extern __shared__ float sh[];", "")
                     + DRIVER)
        subprocess.run(["g++", "-O1", "-shared", "-fPIC", "-I", HERE, "-o", so, path], check=True)
        lib = ctypes.CDLL(so)
        vals = np.zeros(G * npos)
        status = np.zeros(1, np.int32)
        run = lib.host_run
        run.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p,
                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        run(1, P(pk), M * pk.shape[2], G, P(vals), P(status), P(partial), P(lt), P(la))
        assert status[0] == 0
        out.append(vals)
    assert np.array_equal(out[0], out[1])
