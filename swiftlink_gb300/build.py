"""Build the in-tree CUDA library swiftlink_gb300/_build/libswiftlink_gb300.so.

Seven translation units compiled in parallel for sm_103a only, then linked
with the static CUDA runtime and NVRTC (which compiles the problem-specialised
kernels at run time):
  csrc/sl_kernels.cu  (nvcc, -gencode arch=compute_103a,code=sm_103a)
  csrc/sl_noalloc.cu  (nvcc, same flags)
  csrc/sl_host.cc     (g++ against the CUDA runtime headers)
  csrc/sl_jit.cc      (g++, NVRTC source generator and loader)
  csrc/sl_peel.cc     (g++, peel-sequence generator)
  csrc/sl_lsjit.cc    (g++, the L-sampler specialised per pedigree, NVRTC;
                       it embeds csrc/sl_philox.cuh, the Philox shared with
                       sl_kernels.cu, as a string generated into _build)
  csrc/sl_adjjit.cc   (g++, the trait-peel adjoint specialised per pedigree,
                       NVRTC)
and the program swiftlink_gb300/_build/swift_gb300 (csrc/sl_cli.cc, the
LINKAGE-file front end) linked against the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libswiftlink_gb300.so")
CLI = os.path.join(OUT, "swift_gb300")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose: bool = False, force: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    philox = os.path.join(CSRC, "sl_philox.cuh")
    hdrs = [os.path.join(CSRC, "sl_internal.h"), os.path.join(CSRC, "sl_jit.h"), os.path.join(CSRC, "sl_lsjit.h"),
            os.path.join(CSRC, "sl_adjjit.h"), philox, os.path.join(os.path.dirname(HERE), "include", "swiftlink_gb300.h")]
    # the Philox source as a C++ string literal, for the run-time compiled kernels
    inc = os.path.join(OUT, "sl_philox_src.inc")
    if force or _stale(inc, [philox]):
        with open(philox) as f:
            text = f.read()
        with open(inc, "w") as f:
            f.write('R"SLPHILOX(' + text + ')SLPHILOX"\n')
    cu = os.path.join(CSRC, "sl_kernels.cu")
    cu2 = os.path.join(CSRC, "sl_noalloc.cu")
    cc = os.path.join(CSRC, "sl_host.cc")
    jc = os.path.join(CSRC, "sl_jit.cc")
    jc_o = os.path.join(OUT, "sl_jit.o")
    pc = os.path.join(CSRC, "sl_peel.cc")
    pc_o = os.path.join(OUT, "sl_peel.o")
    lj = os.path.join(CSRC, "sl_lsjit.cc")
    lj_o = os.path.join(OUT, "sl_lsjit.o")
    aj = os.path.join(CSRC, "sl_adjjit.cc")
    aj_o = os.path.join(OUT, "sl_adjjit.o")
    cli = os.path.join(CSRC, "sl_cli.cc")
    cli_o = os.path.join(OUT, "sl_cli.o")
    cu_o = os.path.join(OUT, "sl_kernels.o")
    cu2_o = os.path.join(OUT, "sl_noalloc.o")
    cc_o = os.path.join(OUT, "sl_host.o")
    jobs = []
    for src, obj in ((cu, cu_o), (cu2, cu2_o)):
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v", "-c", src, "-o", obj])
    for src, obj in ((cc, cc_o), (jc, jc_o), (pc, pc_o), (cli, cli_o), (lj, lj_o), (aj, aj_o)):
        if force or _stale(obj, [src] + hdrs + ([inc] if src == lj else [])):
            # no contraction of a * b + c into FMA: host FP64 (priors, tempered maps,
            # likelihood sums) must round as the reference's x86-64 build does, on aarch64 too
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off",
                         "-I" + os.path.join(cuda, "include"), "-I" + OUT,
                         "-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, [cu_o, cu2_o, cc_o, jc_o, pc_o, lj_o, aj_o]):
        lib64 = os.path.join(cuda, "lib64")
        logs.append(_run([nvcc, GENCODE, "-shared", "-cudart", "static", "-o", LIB, cu_o, cu2_o, cc_o, jc_o, pc_o, lj_o, aj_o,
                          "-L" + lib64, "-lnvrtc", "-Xlinker", "-rpath=" + lib64]))
    if force or _stale(CLI, [cli_o, LIB]):
        lib64 = os.path.join(cuda, "lib64")
        logs.append(_run(["g++", "-o", CLI, cli_o, "-L" + OUT, "-lswiftlink_gb300",
                          "-Wl,-rpath,$ORIGIN", "-Wl,-rpath-link," + lib64]))
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
