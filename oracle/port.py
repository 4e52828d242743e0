"""TEST INFRASTRUCTURE ONLY: ctypes view of the C restatement (sl_oracle.c).

The library is built by `make -C oracle port` (also run by
__graft_entry__.build()) into oracle/_build/libsloracle.so.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the checker
or as the timed CPU port; the product path never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsloracle.so")

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.slo_fag_likelihood.restype = ctypes.c_double
        _lib.slo_loglik.restype = ctypes.c_double
        _lib.slo_margin.restype = ctypes.c_double
        _lib.slo_philox_uniform.restype = ctypes.c_double
        _lib.slo_philox_uniform.argtypes = [ctypes.c_uint64] * 3
    return _lib


class _Problem(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("N", "F", "M", "K", "n_lod")] + [
        (n, ctypes.c_void_p) for n in (
            "mother", "father", "sex", "geno", "typed", "legal", "prior", "dprob", "theta",
            "partial", "minor", "op_type", "op_peel", "cut_off", "cut", "prev_off", "prev",
            "ch_off", "ch")
    ]


def _csr(lists):
    off = np.zeros(len(lists) + 1, np.int32)
    for i, x in enumerate(lists):
        off[i + 1] = off[i] + len(x)
    flat = np.concatenate([np.asarray(x, np.int32) for x in lists]) if off[-1] else np.zeros(1, np.int32)
    return off, flat.astype(np.int32)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Port:
    """Holds the arrays of one problem (a dict of numpy arrays, see tests/golden)."""

    def __init__(self, prob: dict):
        self.keep = {}
        g = lambda k, dt: self.keep.setdefault(k, np.ascontiguousarray(prob[k], dt))
        self.N, self.F, self.M = int(prob["N"]), int(prob["F"]), int(prob["M"])
        self.K, self.n_lod = int(prob["K"]), int(prob["n_lod"])
        cut_off, cut = _csr(prob["op_cutset"])
        prev_off, prev = _csr(prob["op_prev"])
        ch_off, ch = _csr(prob["op_children"])
        for k, v in dict(cut_off=cut_off, cut=cut, prev_off=prev_off, prev=prev, ch_off=ch_off,
                         ch=ch).items():
            self.keep[k] = v
        s = _Problem()
        s.N, s.F, s.M, s.K, s.n_lod = self.N, self.F, self.M, self.K, self.n_lod
        s.mother = _p(g("mother", np.int32))
        s.father = _p(g("father", np.int32))
        s.sex = _p(g("sex", np.int32))
        s.geno = _p(g("genotypes", np.uint8))
        s.typed = _p(g("typed", np.uint8))
        s.legal = _p(g("legal", np.uint8))
        s.prior = _p(g("trait_prior", np.float64))
        s.dprob = _p(g("disease_prob", np.float64))
        s.theta = _p(g("theta", np.float64))
        s.partial = _p(g("partial", np.float64))
        s.minor = _p(g("minor", np.float64))
        s.op_type = _p(g("op_type", np.int32))
        s.op_peel = _p(g("op_peel", np.int32))
        s.cut_off, s.cut = _p(cut_off), _p(cut)
        s.prev_off, s.prev = _p(prev_off), _p(prev)
        s.ch_off, s.ch = _p(ch_off), _p(ch)
        self.s = s

    def lstep(self, dg, locus, u):
        dg = np.ascontiguousarray(dg, np.int32).copy()
        u = np.ascontiguousarray(u, np.float64)
        used = ctypes.c_int()
        rc = lib().slo_lstep(ctypes.byref(self.s), _p(dg), int(locus), _p(u), u.size, ctypes.byref(used))
        if rc != 0:
            raise RuntimeError(f"slo_lstep failed ({rc})")
        return dg, used.value

    def lsweep(self, dg, u):
        """slo_lsweep: even loci, then odd loci, in one call; u[l] holds locus
        l's draws.  The graph is updated in place (no per-locus copies)."""
        assert dg.dtype == np.int32 and dg.flags.c_contiguous
        u = np.ascontiguousarray(u, np.float64)
        rc = lib().slo_lsweep(ctypes.byref(self.s), _p(dg), _p(u), int(u.shape[1]))
        if rc != 0:
            raise RuntimeError(f"slo_lsweep failed ({rc})")
        return dg

    def lsteps(self, dg, loci, u):
        """slo_lsteps: L-steps at the listed loci in order, in place; u[i] holds
        the i-th listed locus's draws."""
        assert dg.dtype == np.int32 and dg.flags.c_contiguous
        loci = np.ascontiguousarray(loci, np.int32)
        u = np.ascontiguousarray(u, np.float64)
        assert u.shape[0] == loci.size
        rc = lib().slo_lsteps(ctypes.byref(self.s), _p(dg), _p(loci), loci.size, _p(u), int(u.shape[1]))
        if rc != 0:
            raise RuntimeError(f"slo_lsteps failed ({rc})")
        return dg

    def si(self, dg, start, u):
        """One sequential-imputation pass from locus `start`, draws consumed in
        order: (graph, draws used, weight)."""
        dg = np.ascontiguousarray(dg, np.int32).copy()
        u = np.ascontiguousarray(u, np.float64)
        used = ctypes.c_int()
        w = ctypes.c_double()
        rc = lib().slo_si(ctypes.byref(self.s), _p(dg), int(start), _p(u), u.size, ctypes.byref(used),
                          ctypes.byref(w))
        if rc != 0:
            raise RuntimeError(f"slo_si failed ({rc})")
        return dg, used.value, w.value

    def msweep(self, dg, meioses, u):
        dg = np.ascontiguousarray(dg, np.int32).copy()
        meioses = np.ascontiguousarray(meioses, np.int32)
        u = np.ascontiguousarray(u, np.float64)
        used = np.zeros(meioses.size, np.int32)
        rc = lib().slo_msweep(ctypes.byref(self.s), _p(dg), _p(meioses), meioses.size, _p(u), _p(used))
        if rc != 0:
            raise RuntimeError(f"slo_msweep failed ({rc})")
        return dg, used

    def lod(self, dgs, zero_ok=False):
        dgs = np.ascontiguousarray(dgs, np.int32)
        raw = np.zeros((self.M - 1) * self.n_lod)
        cnt = ctypes.c_uint32()
        tp = ctypes.c_double()
        rc = lib().slo_lod_ex(ctypes.byref(self.s), _p(dgs), dgs.shape[0], _p(raw), ctypes.byref(cnt),
                              ctypes.byref(tp), int(zero_ok))
        if rc != 0:
            raise RuntimeError("slo_lod failed")
        return raw, cnt.value, tp.value

    def lod_range(self, dgs, l0, l1, rescale=True, zero_ok=False):
        """slo_lod_range: the scores of intervals [l0, l1) only, plain or
        with per-rfunction power-of-two rescaling."""
        dgs = np.ascontiguousarray(dgs, np.int32)
        raw = np.zeros(max(1, (l1 - l0) * self.n_lod))
        cnt = ctypes.c_uint32()
        tp = ctypes.c_double()
        rc = lib().slo_lod_range(ctypes.byref(self.s), _p(dgs), dgs.shape[0], int(l0), int(l1), int(rescale),
                                 _p(raw), ctypes.byref(cnt), ctypes.byref(tp), int(zero_ok))
        if rc != 0:
            raise RuntimeError(f"slo_lod_range failed ({rc})")
        return raw[:(l1 - l0) * self.n_lod], cnt.value, tp.value

    def fag(self, dg, locus):
        dg = np.ascontiguousarray(dg, np.int32)
        return lib().slo_fag_likelihood(ctypes.byref(self.s), _p(dg), int(locus))

    def loglik(self, dg):
        dg = np.ascontiguousarray(dg, np.int32)
        return lib().slo_loglik(ctypes.byref(self.s), _p(dg))


def margin_reset():
    lib().slo_margin_reset()


def margin() -> float:
    """Smallest |draw - decision boundary| since margin_reset()."""
    return lib().slo_margin()


def msweep_margins(P: "Port", dg, meiosis: int, u):
    """One M-step (reset and step at `meiosis`) on the restatement, returning
    (graph, per-locus margin of the backward draws: 1 where none was taken)."""
    buf = np.ones(P.M)
    lib().slo_margin_log(_p(buf))
    try:
        out, _ = P.msweep(dg, np.array([meiosis], np.int32), np.asarray(u, np.float64).reshape(1, -1))
    finally:
        lib().slo_margin_log(None)
    return out, buf


def derive_priors(genotypes, typed, minor):
    """L-sampler priors [M][N][4] restated from person.cc:224-299 (every person
    takes the founder branch because the cache is filled while parsing,
    pedigree_parser.cc:157) and Snp::init_probs (genetic_map.h:68-87), with
    the reference's operand order: HW total = ((UU + AU) + UA) + AA, person
    total in state-index order."""
    UU, AA, AU, UA = 0, 1, 2, 3
    minor = np.asarray(minor, np.float64)
    ma = 1.0 - minor
    hw = np.zeros((minor.size, 4))
    hw[:, UU] = ma * ma
    hw[:, AU] = minor * ma
    hw[:, UA] = minor * ma
    hw[:, AA] = minor * minor
    tot = ((hw[:, UU] + hw[:, AU]) + hw[:, UA]) + hw[:, AA]
    hw = hw / tot[:, None]
    table = np.zeros((minor.size, 4, 4))
    masks = {0: [1, 1, 1, 1], 1: [0, 0, 1, 1], 2: [1, 0, 0, 0], 3: [0, 1, 0, 0]}
    for g, m in masks.items():
        pr = hw * np.array(m, np.float64)[None, :]
        t = ((pr[:, 0] + pr[:, 1]) + pr[:, 2]) + pr[:, 3]
        table[:, g, :] = pr / t[:, None]
    geno = np.where(np.asarray(typed, bool)[None, :], np.asarray(genotypes) & 3, 0)
    return table[np.arange(minor.size)[:, None], geno, :]


def philox_uniform(key: int, hi: int, lo: int) -> float:
    return lib().slo_philox_uniform(key, hi, lo)


def tempered(prob: dict, t: float) -> dict:
    """The problem as a chain at MC3 temperature t sees it
    (GeneticMap::set_temperature, genetic_map.cc:95-117): theta_t = (t theta) +
    ((1 - t) 0.5) and maf_t likewise, in that operation order; the L-sampler
    priors keep temperature 1 (they are cached while parsing,
    pedigree_parser.cc:157)."""
    d = dict(prob)
    d["theta"] = (t * np.asarray(prob["theta"], np.float64)) + ((1 - t) * 0.5)
    d["minor"] = (t * np.asarray(prob["minor"], np.float64)) + ((1 - t) * 0.5)
    return d
