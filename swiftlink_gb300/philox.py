"""Vectorised numpy Philox4x32-10 (Salmon et al., SC'11) for replaying the
device driver's draw streams on the host (replays and accounting).  Same construction as the
device code: uniform = ((w0 >> 5) * 2^26 + (w1 >> 6)) * 2^-53."""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def uniform(key: int, hi, lo) -> np.ndarray:
    hi = np.asarray(hi, np.uint64)
    lo = np.asarray(lo, np.uint64)
    hi, lo = np.broadcast_arrays(hi, lo)
    c0 = lo & MASK
    c1 = lo >> np.uint64(32)
    c2 = hi & MASK
    c3 = hi >> np.uint64(32)
    k0 = np.uint64(key & 0xFFFFFFFF)
    k1 = np.uint64((key >> 32) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        n0 = (p1 >> np.uint64(32)) ^ c1 ^ k0
        n2 = (p0 >> np.uint64(32)) ^ c3 ^ k1
        c1 = p1 & MASK
        c3 = p0 & MASK
        c0 = n0 & MASK
        c2 = n2 & MASK
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    a = (c0 >> np.uint64(5)).astype(np.float64)
    b = (c1 >> np.uint64(6)).astype(np.float64)
    return (a * 67108864.0 + b) / 9007199254740992.0


def stage_hi(chain: int, it: int, stage: int) -> int:
    return (chain << 40) ^ (it << 4) ^ stage


def lsweep_draws(seed, chain, it, M, stride):
    """[M][stride] draws of one chain's L-sweep (stage 1, unit = locus)."""
    l = np.arange(M, dtype=np.uint64)[:, None]
    k = np.arange(stride, dtype=np.uint64)[None, :]
    return uniform(seed, stage_hi(chain, it, 1), (l << np.uint64(24)) ^ k)


def msweep_draws(seed, chain, it, nm, M):
    """[nm][M] draws of one chain's M-sweep (stage 2, unit = step)."""
    j = np.arange(nm, dtype=np.uint64)[:, None]
    k = np.arange(M, dtype=np.uint64)[None, :]
    return uniform(seed, stage_hi(chain, it, 2), (j << np.uint64(24)) ^ k)


def chooses_l(seed, chain, it, lprob):
    return float(uniform(seed, stage_hi(chain, it, 7), 0)) < lprob


def shuffled(seed, chain, it, base):
    o = list(base)
    hi = stage_hi(chain, it, 3)
    for i in range(len(o) - 1, 0, -1):
        u = float(uniform(seed, hi, i))
        j = min(int(u * (i + 1)), i)
        o[i], o[j] = o[j], o[i]
    return np.array(o, np.int32)


def exchange_draws(seed, it_end):
    """The two uniforms of the MC3 exchange after the spurt ending at `it_end`
    (stage 9): the adjacent pair, then the acceptance."""
    hi = (0x3FF << 40) ^ (it_end << 4) ^ 9
    return float(uniform(seed, hi, 0)), float(uniform(seed, hi, 1))
