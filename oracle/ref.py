"""TEST INFRASTRUCTURE ONLY: ctypes view of oracle/_ref/libswiftref.so.

The library is the reference's own CPU code (compiled from its sources in this
container by oracle/Makefile) plus a harness (oracle/ref_harness.cc).  It is
used to pin the C restatement (oracle/sl_oracle.c) and to write golden
fixtures; it is absent on machines without the reference sources.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libswiftref.so")

_i = ctypes.c_int
_p = ctypes.c_void_p
_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.ref_load.restype = _p
        _lib.ref_load.argtypes = [ctypes.c_char_p] * 3 + [_i, _i, ctypes.c_uint]
        _lib.ref_free.argtypes = [_p]
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class RefProblem:
    """Everything the hot path consumes, as the reference builds it."""

    N: int
    F: int
    M: int
    K: int
    n_lod: int
    mother: np.ndarray
    father: np.ndarray
    sex: np.ndarray
    typed: np.ndarray
    affection: np.ndarray
    n_children: np.ndarray
    genotypes: np.ndarray      # [M][N] uint8 unphased codes
    disease_prob: np.ndarray   # [N][4]
    trait_prior: np.ndarray    # [M][N][4]
    theta: np.ndarray          # [M-1]
    minor: np.ndarray          # [M]
    partial: np.ndarray        # [M-1]
    gpos: np.ndarray           # [M] Morgans
    op_type: np.ndarray
    op_peel: np.ndarray
    op_cutset: list
    op_prev: list
    op_children: list
    op_nlod: np.ndarray
    legal: np.ndarray          # [M][N] 4-bit masks
    meioses: np.ndarray        # non-ignorable meiosis ids
    freq: float
    penetrance: np.ndarray


class Ref:
    def __init__(self, ped: str, map_: str, dat: str, n_lod: int = 5, peel_iters: int = 10000,
                 seed: int = 1):
        self.h = lib().ref_load(ped.encode(), map_.encode(), dat.encode(), n_lod, peel_iters, seed)
        if not self.h:
            raise RuntimeError("reference failed to load the LINKAGE files")
        d = [ctypes.c_int() for _ in range(6)]
        lib().ref_dims(_p(self.h), *[ctypes.byref(x) for x in d])
        self.N, self.F, self.M, self.K, self.n_lod, self.sex_linked = [x.value for x in d]

    def close(self):
        if self.h:
            lib().ref_free(_p(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def dg_shape(self):
        return (self.M, self.N, 2)

    def problem(self) -> RefProblem:
        N, M, K = self.N, self.M, self.K
        L = lib()
        h = _p(self.h)
        mother, father, sex, typed, aff, nch = (np.zeros(N, np.int32) for _ in range(6))
        geno = np.zeros((M, N), np.uint8)
        dprob = np.zeros((N, 4))
        prior = np.zeros((M, N, 4))
        L.ref_pedigree(h, _ptr(mother), _ptr(father), _ptr(sex), _ptr(typed), _ptr(aff),
                       _ptr(geno), _ptr(dprob), _ptr(prior), _ptr(nch))
        theta = np.zeros(M - 1)
        minor = np.zeros(M)
        partial = np.zeros(M - 1)
        gpos = np.zeros(M)
        L.ref_map(h, _ptr(theta), _ptr(minor), _ptr(partial), _ptr(gpos))
        maxc = 64
        typ, peel, clen, plen, chlen, nlod = (np.zeros(K, np.int32) for _ in range(6))
        cut = np.zeros((K, maxc), np.int32)
        prev = np.zeros((K, maxc), np.int32)
        ch = np.zeros((K, maxc), np.int32)
        rc = L.ref_ops(h, maxc, _ptr(typ), _ptr(peel), _ptr(clen), _ptr(cut), _ptr(plen), _ptr(prev),
                       _ptr(chlen), _ptr(ch), _ptr(nlod))
        if rc != 0:
            raise RuntimeError("op list too wide")
        legal = np.zeros((M, N), np.uint8)
        L.ref_legal(h, _ptr(legal))
        mo = np.zeros(2 * N, np.int32)
        nmo = ctypes.c_int()
        L.ref_meiosis_order(h, _ptr(mo), ctypes.byref(nmo))
        freq = ctypes.c_double()
        pen = np.zeros(3)
        L.ref_disease(h, ctypes.byref(freq), _ptr(pen))
        return RefProblem(
            N=N, F=self.F, M=M, K=K, n_lod=self.n_lod, mother=mother, father=father, sex=sex,
            typed=typed, affection=aff, n_children=nch, genotypes=geno, disease_prob=dprob,
            trait_prior=prior, theta=theta, minor=minor, partial=partial, gpos=gpos,
            op_type=typ, op_peel=peel,
            op_cutset=[cut[k, :clen[k]].copy() for k in range(K)],
            op_prev=[prev[k, :plen[k]].copy() for k in range(K)],
            op_children=[ch[k, :chlen[k]].copy() for k in range(K)],
            op_nlod=nlod, legal=legal, meioses=mo[:nmo.value].copy(),
            freq=freq.value, penetrance=pen)

    def initial_dg(self, si_iters: int = 10):
        dg = np.zeros(self.dg_shape, np.int32)
        ll = ctypes.c_double()
        rc = lib().ref_initial_dg(_p(self.h), si_iters, _ptr(dg), ctypes.byref(ll))
        if rc != 0:
            raise RuntimeError("random descent graph failed")
        return dg, ll.value

    def loglik(self, dg: np.ndarray) -> float:
        dg = np.ascontiguousarray(dg, np.int32)
        ll = ctypes.c_double()
        lib().ref_loglik(_p(self.h), _ptr(dg), ctypes.byref(ll))
        return ll.value

    def set_temperature(self, t: float):
        lib().ref_set_temperature(_p(self.h), ctypes.c_double(t))

    def loglik_tempered(self, dg: np.ndarray, t: float) -> float:
        dg = np.ascontiguousarray(dg, np.int32)
        ll = ctypes.c_double()
        lib().ref_loglik_tempered(_p(self.h), _ptr(dg), ctypes.c_double(t), ctypes.byref(ll))
        return ll.value

    def lstep(self, dg: np.ndarray, locus: int, u: np.ndarray):
        dg = np.ascontiguousarray(dg, np.int32).copy()
        u = np.ascontiguousarray(u, np.float64)
        used = ctypes.c_int()
        rc = lib().ref_lstep(_p(self.h), _ptr(dg), locus, _ptr(u), u.size, ctypes.byref(used))
        if rc != 0:
            raise RuntimeError("uniform buffer overrun in lstep")
        return dg, used.value

    def si(self, dg: np.ndarray, start: int, u: np.ndarray):
        dg = np.ascontiguousarray(dg, np.int32).copy()
        u = np.ascontiguousarray(u, np.float64)
        used = ctypes.c_int()
        w = ctypes.c_double()
        rc = lib().ref_si(_p(self.h), _ptr(dg), int(start), _ptr(u), u.size, ctypes.byref(used), ctypes.byref(w))
        if rc != 0:
            raise RuntimeError("uniform buffer overrun in sequential imputation")
        return dg, used.value, w.value

    def msweep(self, dg: np.ndarray, meioses: np.ndarray, u: np.ndarray):
        dg = np.ascontiguousarray(dg, np.int32).copy()
        meioses = np.ascontiguousarray(meioses, np.int32)
        u = np.ascontiguousarray(u, np.float64)
        assert u.size >= meioses.size * self.M
        used = np.zeros(meioses.size, np.int32)
        rc = lib().ref_msweep(_p(self.h), _ptr(dg), _ptr(meioses), meioses.size, _ptr(u), _ptr(used))
        if rc != 0:
            raise RuntimeError("uniform buffer overrun in msweep")
        return dg, used

    def write_table(self, raw: np.ndarray, count: int, trait_prob: float, path: str):
        """The reference's LinkageWriter::write on the given log-sums."""
        raw = np.ascontiguousarray(raw, np.float64)
        assert raw.size == (self.M - 1) * self.n_lod
        rc = lib().ref_write_table(_p(self.h), _ptr(raw), ctypes.c_uint(count), ctypes.c_double(trait_prob),
                                   path.encode())
        if rc != 0:
            raise RuntimeError("LinkageWriter::write failed")

    def lod(self, dgs: np.ndarray):
        dgs = np.ascontiguousarray(dgs, np.int32)
        n = dgs.shape[0]
        raw = np.zeros((self.M - 1) * self.n_lod)
        cnt = ctypes.c_uint()
        tp = ctypes.c_double()
        lib().ref_lod(_p(self.h), _ptr(dgs), n, _ptr(raw), ctypes.byref(cnt), ctypes.byref(tp))
        return raw, cnt.value, tp.value
