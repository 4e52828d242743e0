"""ctypes binding of the swiftlink_gb300 C ABI (include/swiftlink_gb300.h).

This is glue for tests and benchmarks: every computation happens in the CUDA
library; there is no Python or CPU fallback.  Loading fails loudly when the
library has not been built.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libswiftlink_gb300.so")

SL_OK, SL_EINVAL, SL_ECUDA, SL_EZERO, SL_EILLEGAL, SL_ENOMEM, SL_ENODEV = 0, -1, -2, -3, -4, -5, -6
SL_LOD_FP64, SL_LOD_FP32_RESCALED, SL_LOD_FP64_RESCALED = 0, 1, 2
SL_SAMPLER_EXACT, SL_SAMPLER_FAST = 0, 1
SL_LOD_KERNEL_AUTO, SL_LOD_KERNEL_INTERP, SL_LOD_KERNEL_JIT_REG, SL_LOD_KERNEL_JIT_SMEM = 0, 1, 2, 3
SL_LOD_ZERO_OK = 1
SL_LS_KERNEL_GENERIC, SL_LS_KERNEL_SPECIALISED, SL_LS_KERNEL_BACKGROUND, SL_LS_KERNEL_AUTO = 0, 1, 2, 3
SL_LS_KERNEL_GENERIC32, SL_LS_KERNEL_GENERIC16, SL_LS_KERNEL_GENERIC8 = 4, 5, 6
SL_KERNEL_LSAMPLER, SL_KERNEL_MSAMPLER, SL_KERNEL_LOD, SL_KERNEL_LOD_MERGE, SL_KERNEL_OTHER = 0, 1, 2, 3, 4
SL_ADJOINT_WARP, SL_ADJOINT_THREAD, SL_ADJOINT_SPECIALISED = 1, 2, 3
SL_ADJOINT_VARIANTS = 2

EXPORTED = [
    "sl_create", "sl_destroy", "sl_last_error", "sl_set_descent_graphs", "sl_get_descent_graphs",
    "sl_get_trait_priors", "sl_get_legal_masks", "sl_lsampler_loci", "sl_lsampler_sweep",
    "sl_msampler_sweep", "sl_lod_score_chains", "sl_lod_score_graphs", "sl_lod_results",
    "sl_lod_reset", "sl_run", "sl_synchronize", "sl_device_status", "sl_launch_count",
    "sl_version", "sl_get_stream", "sl_profile", "sl_profile_read", "sl_problem_legal_masks",
    "sl_problem_trait_priors", "sl_problem_trait_prob", "sl_trait_backward",
    "sl_problem_trait_backward_eval", "sl_lod_kernel_info", "sl_ls_kernel_info", "sl_set_temperatures", "sl_mc3_stats",
    "sl_chain_loglik", "sl_peel_sequence", "sl_batch_create", "sl_batch_run", "sl_batch_destroy",
    "sl_sequential_imputation", "sl_sequential_imputation_run", "sl_adjoint_memory", "sl_adjoint_info",
    "sl_adjoint_set_form", "sl_adjoint_kernel_info", "sl_problem_adjoint_source", "sl_ls_tuning",
    "sl_problem_lod_source",
]


class SwiftLinkError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_vp = ctypes.c_void_p


class ProblemDesc(ctypes.Structure):
    _fields_ = [
        ("n_members", ctypes.c_int32), ("n_founders", ctypes.c_int32), ("n_markers", ctypes.c_int32),
        ("lod_per_interval", ctypes.c_int32), ("sex_linked", ctypes.c_int32),
        ("mother", _vp), ("father", _vp), ("sex", _vp), ("typed", _vp), ("genotypes", _vp),
        ("legal", _vp), ("disease_prob", _vp), ("theta", _vp), ("partial_theta", _vp),
        ("minor_freq", _vp), ("n_ops", ctypes.c_int32), ("op_type", _vp), ("op_peelnode", _vp),
        ("cutset_off", _vp), ("cutset", _vp), ("prev_off", _vp), ("prev", _vp),
        ("children_off", _vp), ("children", _vp),
        ("affection", _vp), ("disease_freq", ctypes.c_double), ("penetrance", ctypes.c_double * 3),
    ]


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("n_chains", ctypes.c_int32),
                ("lod_precision", ctypes.c_int32), ("sampler_precision", ctypes.c_int32),
                ("lod_kernel", ctypes.c_int32), ("lod_flags", ctypes.c_int32), ("ls_kernel", ctypes.c_int32)]


class RunOptions(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("burnin", ctypes.c_int32),
                ("scoring_period", ctypes.c_int32), ("first_iteration", ctypes.c_int32),
                ("lsampler_prob", ctypes.c_double), ("seed", ctypes.c_uint64),
                ("exchange_period", ctypes.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"swiftlink_gb300 CUDA library not built ({LIB_PATH}); run "
                               "python -c 'import __graft_entry__ as g; g.build()'")
        L = ctypes.CDLL(LIB_PATH)
        L.sl_last_error.restype = ctypes.c_char_p
        L.sl_last_error.argtypes = [_vp]
        L.sl_version.restype = ctypes.c_char_p
        L.sl_launch_count.restype = ctypes.c_int64
        L.sl_launch_count.argtypes = [_vp]
        L.sl_destroy.argtypes = [_vp]
        L.sl_destroy.restype = None
        P = ctypes.POINTER
        L.sl_problem_adjoint_source.argtypes = [P(ProblemDesc), ctypes.c_int32, ctypes.c_int32, ctypes.c_char_p,
                                                ctypes.c_int64, P(ctypes.c_int64), P(ctypes.c_int32),
                                                P(ctypes.c_double)]
        L.sl_problem_lod_source.argtypes = [P(ProblemDesc), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                            ctypes.c_int32, ctypes.c_char_p, ctypes.c_int64, P(ctypes.c_int64),
                                            P(ctypes.c_int32), P(ctypes.c_double)]
        _lib = L
    return _lib


def peel_sequence(mother, father):
    """sl_peel_sequence: (op_type, op_peel, cutsets, prevs, children) of a
    pedigree given in founders-first order (mother/father -1 for founders)."""
    mo = np.ascontiguousarray(mother, np.int32)
    fa = np.ascontiguousarray(father, np.int32)
    n = mo.size
    cap = n * n + 16
    ot = np.zeros(n, np.int32)
    op = np.zeros(n, np.int32)
    offs = [np.zeros(n + 1, np.int32) for _ in range(3)]
    flats = [np.zeros(cap, np.int32) for _ in range(3)]
    rc = lib().sl_peel_sequence(ctypes.c_int32(n), _p(mo), _p(fa), ctypes.c_int32(cap), _p(ot), _p(op),
                                _p(offs[0]), _p(flats[0]), _p(offs[1]), _p(flats[1]), _p(offs[2]), _p(flats[2]))
    if rc != SL_OK:
        raise SwiftLinkError(rc, "peel sequence")
    lists = [[flats[j][offs[j][k]:offs[j][k + 1]].copy() for k in range(n)] for j in range(3)]
    return ot, op, lists[0], lists[1], lists[2]


def _p(a: np.ndarray):
    return a.ctypes.data_as(_vp)


def _csr(lists):
    off = np.zeros(len(lists) + 1, np.int32)
    for i, x in enumerate(lists):
        off[i + 1] = off[i] + len(x)
    flat = (np.concatenate([np.asarray(x, np.int32) for x in lists]) if off[-1]
            else np.zeros(1, np.int32))
    return off, np.ascontiguousarray(flat, np.int32)


@dataclass
class Problem:
    """One pedigree, map and peel sequence in the reference's internal order."""

    N: int
    F: int
    M: int
    n_lod: int
    mother: np.ndarray
    father: np.ndarray
    sex: np.ndarray
    typed: np.ndarray
    genotypes: np.ndarray      # [M][N]
    disease_prob: np.ndarray   # [N][4]
    theta: np.ndarray
    partial: np.ndarray
    minor: np.ndarray
    op_type: np.ndarray
    op_peel: np.ndarray
    op_cutset: list
    op_prev: list
    op_children: list
    legal: Optional[np.ndarray] = None
    affection: Optional[np.ndarray] = None   # [N] 0 unknown, 1 unaffected, 2 affected
    freq: float = 0.0                        # disease-allele frequency
    penetrance: tuple = (0.0, 0.0, 0.0)      # HOMO_U, HETERO, HOMO_A
    keep: dict = field(default_factory=dict)

    @property
    def K(self) -> int:
        return len(self.op_type)

    @classmethod
    def from_arrays(cls, d: dict, with_legal: bool = True) -> "Problem":
        return cls(N=int(d["N"]), F=int(d["F"]), M=int(d["M"]), n_lod=int(d["n_lod"]),
                   mother=d["mother"], father=d["father"], sex=d["sex"], typed=d["typed"],
                   genotypes=d["genotypes"], disease_prob=d["disease_prob"], theta=d["theta"],
                   partial=d["partial"], minor=d["minor"], op_type=d["op_type"],
                   op_peel=d["op_peel"], op_cutset=list(d["op_cutset"]), op_prev=list(d["op_prev"]),
                   op_children=list(d["op_children"]),
                   legal=d.get("legal") if with_legal else None,
                   affection=d.get("affection"), freq=float(d.get("freq", 0.0)),
                   penetrance=tuple(float(x) for x in d.get("penetrance", (0.0, 0.0, 0.0))))

    def desc(self) -> ProblemDesc:
        k = self.keep
        g = lambda name, a, dt: k.setdefault(name, np.ascontiguousarray(a, dt))
        s = ProblemDesc()
        s.n_members, s.n_founders, s.n_markers = self.N, self.F, self.M
        s.lod_per_interval, s.sex_linked = self.n_lod, 0
        s.mother = _p(g("mother", self.mother, np.int32))
        s.father = _p(g("father", self.father, np.int32))
        s.sex = _p(g("sex", self.sex, np.int32))
        s.typed = _p(g("typed", self.typed, np.uint8))
        s.genotypes = _p(g("genotypes", self.genotypes, np.uint8))
        s.legal = _p(g("legal", self.legal, np.uint8)) if self.legal is not None else None
        s.disease_prob = _p(g("dprob", self.disease_prob, np.float64))
        s.theta = _p(g("theta", self.theta, np.float64))
        s.partial_theta = _p(g("partial", self.partial, np.float64))
        s.minor_freq = _p(g("minor", self.minor, np.float64))
        s.n_ops = self.K
        s.op_type = _p(g("op_type", self.op_type, np.int32))
        s.op_peelnode = _p(g("op_peel", self.op_peel, np.int32))
        for name, lists in (("cutset", self.op_cutset), ("prev", self.op_prev),
                            ("children", self.op_children)):
            off, flat = _csr(lists)
            k[name + "_off"], k[name] = off, flat
        s.cutset_off, s.cutset = _p(k["cutset_off"]), _p(k["cutset"])
        s.prev_off, s.prev = _p(k["prev_off"]), _p(k["prev"])
        s.children_off, s.children = _p(k["children_off"]), _p(k["children"])
        if self.affection is not None:
            s.affection = _p(g("affection", self.affection, np.int32))
            s.disease_freq = self.freq
            for i in range(3):
                s.penetrance[i] = self.penetrance[i]
        s._arrays = k   # the descriptor's pointers stay valid while it lives, even past this Problem
        return s


class Context:
    """A device context holding one problem and n_chains descent graphs."""

    def __init__(self, problem: Problem, n_chains: int = 1, lod_precision: int = SL_LOD_FP64,
                 device: int = 0, sampler_precision: int = SL_SAMPLER_EXACT, lod_kernel: int = SL_LOD_KERNEL_AUTO,
                 lod_flags: int = 0, ls_kernel: int = SL_LS_KERNEL_GENERIC):
        self.problem = problem
        self._desc = problem.desc()
        opt = Options(device, n_chains, lod_precision, sampler_precision, lod_kernel, lod_flags, ls_kernel)
        h = _vp()
        rc = lib().sl_create(ctypes.byref(self._desc), ctypes.byref(opt), ctypes.byref(h))
        if rc != SL_OK:
            raise SwiftLinkError(rc, lib().sl_last_error(None).decode())
        self.h = h
        self.n_chains = n_chains
        self.N, self.F, self.M, self.K = problem.N, problem.F, problem.M, problem.K

    def close(self):
        if getattr(self, "h", None):
            lib().sl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != SL_OK:
            raise SwiftLinkError(rc, lib().sl_last_error(self.h).decode())

    @property
    def launches(self) -> int:
        return lib().sl_launch_count(self.h)

    def set_graphs(self, dgs: np.ndarray, first: int = 0):
        dgs = np.ascontiguousarray(dgs, np.int32).reshape(-1, self.M, self.N, 2)
        self._check(lib().sl_set_descent_graphs(self.h, first, dgs.shape[0], _p(dgs)))

    def get_graphs(self, first: int = 0, n: Optional[int] = None, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Graphs of chains [first, first + n) in the reference's int32 layout,
        into `out` when given (C-contiguous int32 [n][M][N][2])."""
        if out is not None:
            assert out.dtype == np.int32 and out.flags.c_contiguous
            n = out.size // (self.M * self.N * 2)
        n = self.n_chains - first if n is None else n
        if out is None:
            out = np.empty((n, self.M, self.N, 2), np.int32)
        self._check(lib().sl_get_descent_graphs(self.h, first, n, _p(out)))
        return out

    def trait_priors(self) -> np.ndarray:
        out = np.zeros((self.M, self.N, 4))
        self._check(lib().sl_get_trait_priors(self.h, _p(out)))
        return out

    def legal_masks(self) -> np.ndarray:
        out = np.zeros((self.M, self.N), np.uint8)
        self._check(lib().sl_get_legal_masks(self.h, _p(out)))
        return out

    def lsampler_loci(self, loci: Sequence[int], u: np.ndarray, first: int = 0, n_chains: int = 1):
        """u: [n_chains][M][stride] draws."""
        loci = np.ascontiguousarray(loci, np.int32)
        u = np.ascontiguousarray(u, np.float64)
        assert u.ndim == 3 and u.shape[1] == self.M
        self._check(lib().sl_lsampler_loci(self.h, first, n_chains, _p(loci), loci.size, _p(u),
                                           ctypes.c_int64(u.shape[1] * u.shape[2]),
                                           ctypes.c_int64(u.shape[2])))

    def lsampler_sweep(self, u: np.ndarray, first: int = 0, n_chains: int = 1):
        u = np.ascontiguousarray(u, np.float64)
        assert u.ndim == 3 and u.shape[1] == self.M
        self._check(lib().sl_lsampler_sweep(self.h, first, n_chains, _p(u),
                                            ctypes.c_int64(u.shape[1] * u.shape[2]),
                                            ctypes.c_int64(u.shape[2])))

    def msampler_sweep(self, meioses: Sequence[int], u: np.ndarray, first: int = 0, n_chains: int = 1):
        """u: [n_chains][len(meioses)][M] draws."""
        m = np.ascontiguousarray(meioses, np.int32)
        u = np.ascontiguousarray(u, np.float64)
        assert u.ndim == 3 and u.shape[1] == m.size and u.shape[2] == self.M
        self._check(lib().sl_msampler_sweep(self.h, first, n_chains, _p(m), m.size, _p(u),
                                            ctypes.c_int64(u.shape[1] * u.shape[2])))

    def lod_score_chains(self, first: int = 0, n_chains: Optional[int] = None):
        n = self.n_chains - first if n_chains is None else n_chains
        self._check(lib().sl_lod_score_chains(self.h, first, n))

    def lod_score_graphs(self, dgs: np.ndarray):
        dgs = np.ascontiguousarray(dgs, np.int32).reshape(-1, self.M, self.N, 2)
        self._check(lib().sl_lod_score_graphs(self.h, dgs.shape[0], _p(dgs)))

    def lod_results(self):
        raw = np.zeros((self.M - 1) * self.problem.n_lod)
        cnt = ctypes.c_uint64()
        tp = ctypes.c_double()
        self._check(lib().sl_lod_results(self.h, _p(raw), ctypes.byref(cnt), ctypes.byref(tp)))
        return raw, cnt.value, tp.value

    def lod_reset(self):
        self._check(lib().sl_lod_reset(self.h))

    def ls_tuning(self):
        """(lanes per task of the generic L-sampler in use, 0 for the
        specialised one; the autotuner's timed half-sweeps in ms for 32, 16
        and 8 lanes and the specialised kernel, 0 where not timed)."""
        lanes = ctypes.c_int32()
        t = (ctypes.c_double * 4)()
        self._check(lib().sl_ls_tuning(self.h, ctypes.byref(lanes), t))
        return lanes.value, list(t)

    def ls_kernel_info(self):
        """(SL_LS_KERNEL_GENERIC or SL_LS_KERNEL_SPECIALISED in use, milliseconds spent compiling it;
        -1 while a background compile runs)."""
        k = ctypes.c_int32()
        ms = ctypes.c_double()
        self._check(lib().sl_ls_kernel_info(self.h, ctypes.byref(k), ctypes.byref(ms)))
        return k.value, ms.value

    def lod_kernel_info(self):
        """(SL_LOD_KERNEL_* in use, milliseconds spent compiling specialised forms)."""
        k = ctypes.c_int32()
        ms = ctypes.c_double()
        self._check(lib().sl_lod_kernel_info(self.h, ctypes.byref(k), ctypes.byref(ms)))
        return k.value, ms.value

    def adjoint_memory(self, bytes_per_task: int = 0):
        """Plan the trait-peel adjoint within bytes_per_task of shared memory
        per task (0: the default); returns (segments, bytes used per task):
        one segment keeps every rfunction, more recompute them."""
        seg = ctypes.c_int32()
        used = ctypes.c_int64()
        self._check(lib().sl_adjoint_memory(self.h, ctypes.c_int64(bytes_per_task), ctypes.byref(seg),
                                            ctypes.byref(used)))
        return seg.value, used.value

    def adjoint_info(self):
        """(SL_ADJOINT_WARP / _THREAD / _SPECIALISED or 0 before the first
        call, the timed launch of the warp, thread and specialised forms in ms,
        0 for a form not timed)."""
        f = ctypes.c_int32()
        a = ctypes.c_double()
        b = ctypes.c_double()
        c = ctypes.c_double()
        self._check(lib().sl_adjoint_info(self.h, ctypes.byref(f), ctypes.byref(a), ctypes.byref(b),
                                          ctypes.byref(c)))
        return f.value, a.value, b.value, c.value

    def adjoint_set_form(self, form: int = 0, variant: int = 0):
        """Fix the adjoint's form (SL_ADJOINT_*; for SL_ADJOINT_SPECIALISED
        also its variant), or 0 to choose by timing."""
        self._check(lib().sl_adjoint_set_form(self.h, ctypes.c_int32(form), ctypes.c_int32(variant)))

    def adjoint_kernel_info(self):
        """(operation shapes, variant in use, its registers per thread,
        compile ms of the variants) of the specialised adjoint; compile ms 0
        before it was needed, -1 if it did not build."""
        n = ctypes.c_int32()
        v = ctypes.c_int32()
        r = ctypes.c_int32()
        ms = ctypes.c_double()
        self._check(lib().sl_adjoint_kernel_info(self.h, ctypes.byref(n), ctypes.byref(v), ctypes.byref(r),
                                                 ctypes.byref(ms)))
        return n.value, v.value, r.value, ms.value

    def trait_backward(self, dgs: Optional[np.ndarray] = None):
        """d log L / d (theta_L, theta_R, pen x3, frequency) at every LOD
        position of every graph: [G][M-1][n][6], and d log P(T) / d (pen x3,
        frequency): [4]."""
        n = self.problem.n_lod
        pt = np.zeros(4)
        if dgs is None:
            self._check(lib().sl_trait_backward(self.h, 0, None, None, _p(pt)))
            return None, pt
        dgs = np.ascontiguousarray(dgs, np.int32).reshape(-1, self.M, self.N, 2)
        grad = np.zeros((dgs.shape[0], self.M - 1, n, 6))
        self._check(lib().sl_trait_backward(self.h, dgs.shape[0], _p(dgs), _p(grad), _p(pt)))
        return grad, pt

    def run(self, iterations: int, burnin: int = 0, period: int = 10, lprob: float = 0.5,
            seed: int = 1, first_iteration: int = 0, exchange_period: int = 0):
        o = RunOptions(iterations, burnin, period, first_iteration, lprob, seed, exchange_period)
        self._check(lib().sl_run(self.h, ctypes.byref(o)))

    def set_temperatures(self, temps):
        t = np.ascontiguousarray(temps, np.float64)
        assert t.shape == (self.n_chains,)
        self._check(lib().sl_set_temperatures(self.h, _p(t)))

    def mc3_stats(self):
        n = max(1, self.n_chains - 1)
        acc = np.zeros(n, np.int64)
        prop = np.zeros(n, np.int64)
        self._check(lib().sl_mc3_stats(self.h, _p(acc), _p(prop)))
        return acc[: self.n_chains - 1], prop[: self.n_chains - 1]

    def sequential_imputation(self, starts, draws, first: int = 0):
        """One imputation pass per chain from the given start loci, draws [n][L]
        consumed in order; returns the passes' weights."""
        st = np.ascontiguousarray(starts, np.int32)
        u = np.ascontiguousarray(draws, np.float64)
        n = st.size
        assert u.ndim == 2 and u.shape[0] == n
        w = np.zeros(n)
        self._check(lib().sl_sequential_imputation(self.h, first, n, _p(st), _p(u), ctypes.c_int64(u.shape[1]),
                                                   _p(w)))
        return w

    def sequential_imputation_run(self, iterations: int, seed: int = 1):
        w = np.zeros(self.n_chains)
        self._check(lib().sl_sequential_imputation_run(self.h, int(iterations), ctypes.c_uint64(seed), _p(w)))
        return w

    def chain_loglik(self, graph_chain: int, map_chain: int) -> float:
        v = ctypes.c_double()
        self._check(lib().sl_chain_loglik(self.h, int(graph_chain), int(map_chain), ctypes.byref(v)))
        return v.value

    def stream_handle(self) -> int:
        h = _vp()
        self._check(lib().sl_get_stream(self.h, ctypes.byref(h)))
        return h.value or 0

    def profile(self, enable: bool):
        self._check(lib().sl_profile(self.h, 1 if enable else 0))

    def profile_read(self, kernel: int):
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        self._check(lib().sl_profile_read(self.h, kernel, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def synchronize(self):
        self._check(lib().sl_synchronize(self.h))

    def status(self) -> int:
        st = ctypes.c_int32()
        self._check(lib().sl_device_status(self.h, ctypes.byref(st)))
        return st.value


def lod_table(raw: np.ndarray, count: int, trait_prob: float) -> np.ndarray:
    """LODscores::get (lod_score.h:86-88): (raw - ln count - P(T)) / ln 10."""
    return (raw - np.log(count) - trait_prob) / np.log(10.0)


class Batch:
    """Several contexts run by one graph launch per spurt (sl_batch_*)."""

    def __init__(self, contexts):
        self.contexts = list(contexts)
        arr = (_vp * len(self.contexts))(*[c.h for c in self.contexts])
        h = _vp()
        rc = lib().sl_batch_create(arr, len(self.contexts), ctypes.byref(h))
        if rc != SL_OK:
            raise SwiftLinkError(rc, lib().sl_last_error(None).decode())
        self.h = h

    def run(self, iterations: int, burnin: int = 0, period: int = 10, lprob: float = 0.5, seed: int = 1,
            first_iteration: int = 0, exchange_period: int = 0):
        o = RunOptions(iterations, burnin, period, first_iteration, lprob, seed, exchange_period)
        rc = lib().sl_batch_run(self.h, ctypes.byref(o))
        if rc != SL_OK:
            raise SwiftLinkError(rc, lib().sl_last_error(None).decode())

    def close(self):
        if getattr(self, "h", None):
            lib().sl_batch_destroy.argtypes = [_vp]
            lib().sl_batch_destroy.restype = None
            lib().sl_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
