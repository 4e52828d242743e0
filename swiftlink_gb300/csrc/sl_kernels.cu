// sm_103a kernels for the SwiftLink MCMC hot path.
//
//  * lsampler_kernel   -- L-sampler, one warp per (chain, locus), FP64 with the
//                         reference's operation order (bit-exact decisions).
//  * msampler_kernel   -- M-sampler sweep, one block per chain: founder-allele
//                         graph likelihoods in parallel over loci, then a
//                         warp-wide serial forward-filter / backward-sample.
//  * lod_kernel<T,R>   -- trait peel at every (graph, interval, position), one
//                         warp per task; T=double is the plain FP64 form,
//                         T=float with R=true rescales every rfunction by a
//                         power of two and carries the exponent.
//  * lod_merge_kernel  -- FP64 log-sum accumulation into the LOD table.
//
// FP64 arithmetic on decision paths uses __dmul_rn/__dadd_rn/__ddiv_rn so no
// multiply-add is contracted and the doubles match the reference's.

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "sl_internal.h"

namespace sl {

#define DMUL __dmul_rn
#define DADD __dadd_rn
#define DSUB __dsub_rn
#define DDIV __ddiv_rn
#define FULLMASK 0xffffffffu

__device__ __forceinline__ int dgbit(const uint32_t* col, int b) { return (col[b >> 5] >> (b & 31)) & 1; }
__device__ __forceinline__ int digit(int ext, int pos) { return (ext >> (2 * pos)) & 3; }
__device__ __forceinline__ void set_status(int* st, int code) { atomicCAS(st, 0, code); }

// maternal / paternal allele of a phased state: U=0, A=1
__device__ __forceinline__ int mat_allele(int s) { return (s == AA || s == AU) ? 1 : 0; }
__device__ __forceinline__ int pat_allele(int s) { return (s == AA || s == UA) ? 1 : 0; }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11): counter-based uniform in [0, 1).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double philox_u01(uint64_t key, uint64_t c_hi, uint64_t c_lo) {
    uint32_t c0 = (uint32_t)c_lo, c1 = (uint32_t)(c_lo >> 32);
    uint32_t c2 = (uint32_t)c_hi, c3 = (uint32_t)(c_hi >> 32);
    uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c1 = lo1;
        c3 = lo0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    uint64_t hi = c0 >> 5, lo = c1 >> 6;
    return (double)(hi * 67108864ull + lo) * (1.0 / 9007199254740992.0);
}

// Where uniform draws come from: a caller-supplied array (bit-exact replay of
// the reference) or the Philox stream (device-driven runs).  `unit` is the
// locus (L-sampler) or the meiosis step (M-sampler) within the sweep.
struct Draws {
    const double* u;
    int64_t chain_stride, unit_stride;
    uint64_t seed, iter;
    int stage;
    __device__ __forceinline__ double get(int chain_rel, int chain, int64_t unit, int64_t k) const {
        if (u) return u[chain_rel * chain_stride + unit * unit_stride + k];
        uint64_t hi = ((uint64_t)chain << 40) ^ (iter << 4) ^ (uint64_t)stage;
        return philox_u01(seed, hi, ((uint64_t)unit << 24) ^ (uint64_t)k);
    }
};

// ---------------------------------------------------------------------------
// L-sampler
// ---------------------------------------------------------------------------

// Recombination distributions of one child's two meioses for every parental
// state (SamplerRfunction::get_recombination_distribution,
// sampler_rfunction.cc:102-157): d[side*8 + state*2 + allele].
__device__ void ls_dist_one(const ProblemDev& P, int person, const uint32_t* colL, const uint32_t* colR,
                            int l, double th, double an, double th2, double an2, double* d) {
    for (int side = 0; side < 2; ++side) {
        const int b = 2 * (person - P.F) + side;
        double* s = d + side * 8;
        s[UU * 2 + 0] = 1.0; s[UU * 2 + 1] = 0.0;
        s[AA * 2 + 0] = 0.0; s[AA * 2 + 1] = 1.0;
        double tmp0 = 0.5, tmp1 = 0.5;
        if (l != 0) {
            const bool cross = dgbit(colL, b) != 0;
            tmp0 = DMUL(tmp0, cross ? th2 : an2);
            tmp1 = DMUL(tmp1, cross ? an2 : th2);
        }
        if (l != P.M - 1) {
            const bool cross = dgbit(colR, b) != 0;
            tmp0 = DMUL(tmp0, cross ? th : an);
            tmp1 = DMUL(tmp1, cross ? an : th);
        }
        const double total = DADD(tmp0, tmp1);
        const double uau = DDIV(tmp1, total);
        s[AU * 2 + 0] = uau;
        s[AU * 2 + 1] = DSUB(1.0, uau);
        const double uua = DDIV(tmp0, total);
        s[UA * 2 + 0] = uua;
        s[UA * 2 + 1] = DSUB(1.0, uua);
    }
}

__device__ __forceinline__ void ls_dists(const ProblemDev& P, const OpDev& op, const uint32_t* colL,
                                         const uint32_t* colR, int l, double th, double an, double th2,
                                         double an2, double* dist, int lane) {
    const int nch = op.type == CHILD ? 1 : (op.type == PARENT ? op.n_child : 0);
    if (lane < nch) {
        const int person = op.type == CHILD ? op.peel : P.opdata[op.child_at + 4 * lane];
        ls_dist_one(P, person, colL, colR, l, th, an, th2, an2, dist + 16 * lane);
    }
}

__device__ __forceinline__ bool ls_valid(const int32_t* cut, int c, const uint8_t* gcol, int cell) {
    bool ok = true;
    for (int q = 0; q < c; ++q) ok &= ((gcol[cut[q]] >> (4 + digit(cell, q))) & 1) != 0;
    return ok;
}

// One presum entry (cell, peel state v) in the reference's product order
// (sampler_rfunction.cc:190-287, rfunction.cc:116-142).
__device__ double ls_term(const ProblemDev& P, const OpDev& op, const double* A, const double* dist,
                          int cell, int v, double tv) {
    const int ext = cell | (v << (2 * op.c));
    double tmp = tv;
    if (op.type == CHILD) {
        const int mt = digit(ext, op.mpos), pt = digit(ext, op.fpos);
        const double T = DMUL(dist[mt * 2 + mat_allele(v)], dist[8 + pt * 2 + pat_allele(v)]);
        tmp = DMUL(tmp, T);
    }
    const int32_t* pd = P.opdata + op.prev_at;
    for (int j = 0; j < op.n_prev; ++j) {
        const int moff = pd[0], pc = pd[1];
        int idx = 0;
        for (int q = 0; q < pc; ++q) idx |= digit(ext, pd[2 + q]) << (2 * q);
        tmp = DMUL(tmp, A[moff + idx]);
        pd += 2 + pc;
    }
    if (op.type == PARENT) {
        double cp = 1.0;
        const int32_t* cd = P.opdata + op.child_at;
        for (int c = 0; c < op.n_child; ++c, cd += 4) {
            const int kt = digit(ext, cd[1]), other = digit(ext, cd[2]);
            const int mt = cd[3] ? v : other, pt = cd[3] ? other : v;
            const double T = DMUL(dist[c * 16 + mt * 2 + mat_allele(kt)],
                                  dist[c * 16 + 8 + pt * 2 + pat_allele(kt)]);
            cp = DMUL(cp, T);
        }
        tmp = DMUL(tmp, cp);
    }
    return tmp;
}

__device__ __forceinline__ size_t ls_warp_bytes(const ProblemDev& P) {
    return (size_t)P.arena * 8 + (size_t)P.max_child * 128 + (((size_t)P.N + 15) & ~(size_t)15);
}

// One warp per (chain, locus) task; the listed loci must be pairwise
// non-adjacent so each task owns its descent-graph column.
__global__ void __launch_bounds__(128) lsampler_kernel(ProblemDev P, uint32_t* dg, int first, int nchain,
                                                       const int32_t* loci, int nloci, Draws draws,
                                                       const uint8_t* sel, int want, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* base = smem + (size_t)warp * ls_warp_bytes(P);
    double* A = (double*)base;
    double* dist = A + P.arena;
    int8_t* assign = (int8_t*)(dist + 16 * P.max_child);
    const int64_t ntask = (int64_t)nchain * nloci;
    for (int64_t t = (int64_t)blockIdx.x * wpb + warp; t < ntask; t += (int64_t)gridDim.x * wpb) {
        const int cr = (int)(t / nloci);
        if (sel && sel[cr] != want) continue;
        const int chain = first + cr;
        const int l = loci[t % nloci];
        uint32_t* colC = dg + ((size_t)chain * P.M + l) * P.W;
        const uint32_t* colL = l > 0 ? colC - P.W : nullptr;
        const uint32_t* colR = l < P.M - 1 ? colC + P.W : nullptr;
        double th = 1.0, an = 1.0, th2 = 1.0, an2 = 1.0;
        if (l > 0) { th2 = P.theta[l - 1]; an2 = DSUB(1.0, th2); }
        if (l < P.M - 1) { th = P.theta[l]; an = DSUB(1.0, th); }
        const uint8_t* gcol = P.geno + (size_t)l * P.N;
        const double* pri = P.prior + (size_t)l * 16;
        // forward peel over the valid cells of every rfunction
        for (int k = 0; k < P.K; ++k) {
            const OpDev op = P.ops[k];
            ls_dists(P, op, colL, colR, l, th, an, th2, an2, dist, lane);
            __syncwarp();
            const int ncell = 1 << (2 * op.c);
            const int32_t* cut = P.opdata + op.cut_at;
            const double* trait = pri + 4 * (gcol[op.peel] & 3);
            double* out = A + op.mat_off;
            for (int cell = lane; cell < ncell; cell += 32) {
                double total = 0.0;
                if (ls_valid(cut, op.c, gcol, cell)) {
                    for (int v = 0; v < 4; ++v) {
                        const double tv = trait[v];
                        if (tv == 0.0) continue;
                        total = DADD(total, ls_term(P, op, A, dist, cell, v, tv));
                    }
                }
                out[cell] = total;
            }
            __syncwarp();
        }
        const double root = A[P.ops[P.K - 1].mat_off];
        if (root == 0.0) {
            if (lane == 0) set_status(status, ST_ZERO_LIK);
            __syncwarp();
            continue;
        }
        for (int i = lane; i < P.N; i += 32) assign[i] = -1;
        __syncwarp();
        // backward sampling of ordered genotypes (SamplerRfunction::sample)
        for (int k = P.K - 1; k >= 0; --k) {
            const OpDev op = P.ops[k];
            ls_dists(P, op, colL, colR, l, th, an, th2, an2, dist, lane);
            __syncwarp();
            const int32_t* cut = P.opdata + op.cut_at;
            const double* trait = pri + 4 * (gcol[op.peel] & 3);
            int cellidx = 0;
            bool known = true;
            for (int q = 0; q < op.c; ++q) {
                const int a = assign[cut[q]];
                known &= a >= 0;
                cellidx |= (a & 3) << (2 * q);
            }
            double pv = 0.0;
            if (lane < 4 && known) {
                const double tv = trait[lane];
                if (tv != 0.0 && ls_valid(cut, op.c, gcol, cellidx)) pv = ls_term(P, op, A, dist, cellidx, lane, tv);
            }
            const double p0 = __shfl_sync(FULLMASK, pv, 0), p1 = __shfl_sync(FULLMASK, pv, 1);
            const double p2 = __shfl_sync(FULLMASK, pv, 2), p3 = __shfl_sync(FULLMASK, pv, 3);
            if (lane == 0) {
                if (!known) set_status(status, ST_ILLEGAL_DG);
                double pd[4] = {p0, p1, p2, p3};
                const double tot = DADD(DADD(DADD(p0, p1), p2), p3);
                if (tot != 0.0)
                    for (int v = 0; v < 4; ++v) pd[v] = DDIV(pd[v], tot);
                const double r = draws.get(cr, chain, l, P.K - 1 - k);
                double acc = 0.0;
                int lastv = 0, pick = -1;
                for (int v = 0; v < 4; ++v) {
                    acc = DADD(acc, pd[v]);
                    if (r < acc) { pick = v; break; }
                    if (pd[v] != 0.0) lastv = v;
                }
                assign[op.peel] = (int8_t)(pick >= 0 ? pick : lastv);
            }
            __syncwarp();
        }
        // meiosis indicators (locus_sampler2.cc:32-125), person order, maternal first
        if (lane == 0) {
            int64_t cursor = P.K;
            for (int i = P.F; i < P.N; ++i) {
                const int tr = assign[i];
                for (int par = 0; par < 2; ++par) {
                    const int ptr = assign[par == 0 ? P.mother[i] : P.father[i]];
                    const int allele = par == 0 ? ((tr == UU || tr == UA) ? 0 : 1) : ((tr == UU || tr == AU) ? 0 : 1);
                    int mi;
                    const int b = 2 * (i - P.F) + par;
                    if (ptr == UA || ptr == AU) {
                        mi = allele == 0 ? (ptr == UA ? 0 : 1) : (ptr == UA ? 1 : 0);
                    } else {
                        double p0 = 1.0, p1 = 1.0;
                        if (l != 0) {
                            const int d = dgbit(colL, b);
                            p0 = DMUL(p0, d == 0 ? an2 : th2);
                            p1 = DMUL(p1, d == 1 ? an2 : th2);
                        }
                        if (l != P.M - 1) {
                            const int d = dgbit(colR, b);
                            p0 = DMUL(p0, d == 0 ? an : th);
                            p1 = DMUL(p1, d == 1 ? an : th);
                        }
                        const double r = draws.get(cr, chain, l, cursor++);
                        mi = (r < DDIV(p0, DADD(p0, p1))) ? 0 : 1;
                    }
                    uint32_t w = colC[b >> 5];
                    w = (w & ~(1u << (b & 31))) | ((uint32_t)mi << (b & 31));
                    colC[b >> 5] = w;
                }
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Founder allele graph likelihood (FounderAlleleGraph4::likelihood,
// founder_allele_graph4.cc:34-442), one thread, state in shared memory.
// ---------------------------------------------------------------------------
struct FagState {
    double* pr0;      // [2F] prob[0][group]
    double* pr1;      // [2F]
    int16_t* edge;    // [2N]
    int16_t* member;  // [2F]
    int8_t* fixed;    // [2F]
    uint8_t* active;  // [2F]
    uint8_t* a0;      // [2F] allele_assignment[0][founder allele]
    uint8_t* a1;      // [2F]
};

__host__ __device__ inline int fag_state_bytes(int N, int F) {
    int b = 2 * F * 16 + 2 * N * 2 + 2 * F * 2 + 2 * F * 4;
    return (b + 15) & ~15;
}

__device__ __forceinline__ FagState fag_bind(unsigned char* p, int N, int F) {
    FagState s;
    s.pr0 = (double*)p;
    s.pr1 = s.pr0 + 2 * F;
    s.edge = (int16_t*)(s.pr1 + 2 * F);
    s.member = s.edge + 2 * N;
    s.fixed = (int8_t*)(s.member + 2 * F);
    s.active = (uint8_t*)(s.fixed + 2 * F);
    s.a0 = s.active + 2 * F;
    s.a1 = s.a0 + 2 * F;
    return s;
}

__device__ __forceinline__ int fag_legal(int obs, int x, int y) {
    if (obs == G_HETERO) return x != y;
    if (obs == G_HOMOZ_A) return x == G_HOMOZ_A && y == G_HOMOZ_A;
    return x == G_HOMOZ_B && y == G_HOMOZ_B;
}

__device__ __forceinline__ int fag_other(int obs, int x) {
    if (obs == G_HETERO) return x == G_HOMOZ_A ? G_HOMOZ_B : G_HOMOZ_A;
    if (obs == G_HOMOZ_A) return x == G_HOMOZ_A ? G_HOMOZ_A : G_UNTYPED;
    return x == G_HOMOZ_B ? G_HOMOZ_B : G_UNTYPED;
}

__device__ void fag_combine(FagState& s, int nfa, int c1, int c2, bool flip) {
    for (int i = 0; i < nfa; ++i) {
        if (s.member[i] == c2) {
            s.member[i] = (int16_t)c1;
            if (flip) { uint8_t t = s.a0[i]; s.a0[i] = s.a1[i]; s.a1[i] = t; }
        }
    }
    if (flip) {
        s.pr0[c1] = DMUL(s.pr0[c1], s.pr1[c2]);
        s.pr1[c1] = DMUL(s.pr1[c1], s.pr0[c2]);
    } else {
        s.pr0[c1] = DMUL(s.pr0[c1], s.pr0[c2]);
        s.pr1[c1] = DMUL(s.pr1[c1], s.pr1[c2]);
    }
    s.active[c2] = 0;
}

// Edges of the column (FounderAlleleGraph4::reset, founder_allele_graph4.cc:
// 543-569) with one meiosis optionally toggled, which equals flip() and its
// propagation (founder_allele_graph4.cc:571-597).
__device__ void fag_edges(const ProblemDev& P, const uint32_t* col, FagState& s, int flip_b) {
    for (int n = 0; n < P.N; ++n) {
        const int pid = P.fag_order[n];
        if (pid < P.F) {
            s.edge[2 * pid] = (int16_t)(2 * pid);
            s.edge[2 * pid + 1] = (int16_t)(2 * pid + 1);
        } else {
            const int b = 2 * (pid - P.F);
            const int vm = dgbit(col, b) ^ (flip_b == b);
            const int vp = dgbit(col, b + 1) ^ (flip_b == b + 1);
            s.edge[2 * pid] = s.edge[2 * P.mother[pid] + vm];
            s.edge[2 * pid + 1] = s.edge[2 * P.father[pid] + vp];
        }
    }
}

#define ASG(s, w, fa) ((w) == 0 ? (s).a0[fa] : (s).a1[fa])
#define PRB(s, w, g) (*((w) == 0 ? &(s).pr0[g] : &(s).pr1[g]))

__device__ double fag_like(const ProblemDev& P, int locus, FagState& s) {
    const int nfa = 2 * P.F;
    const double minor = P.minor[locus];
    const double major = DSUB(1.0, minor);
    for (int i = 0; i < nfa; ++i) {
        s.member[i] = -1; s.fixed[i] = -1; s.active[i] = 0; s.a0[i] = 0; s.a1[i] = 0;
    }
    int gi = 0;
    const uint8_t* gcol = P.geno + (size_t)locus * P.N;
#define FREQ(g) ((g) == G_HOMOZ_A ? major : minor)
    for (int i = 0; i < P.N; ++i) {
        if (!P.typed[i]) continue;
        const int g = gcol[i] & 3;
        if (g == G_UNTYPED) continue;
        const int mfa = s.edge[2 * i], pfa = s.edge[2 * i + 1];
        if (mfa == pfa) {
            if (g == G_HETERO) return 0.0;
            const int g1 = s.member[mfa];
            if (g1 != -1) {
                const int f1 = s.fixed[g1];
                if (f1 != -1) {
                    if (g != ASG(s, f1, mfa)) return 0.0;
                } else {
                    if (s.a0[mfa] == g) { s.fixed[g1] = 0; s.pr1[g1] = 0.0; }
                    else if (s.a1[mfa] == g) { s.fixed[g1] = 1; s.pr0[g1] = 0.0; }
                    else return 0.0;
                }
            } else {
                s.member[mfa] = (int16_t)gi; s.fixed[gi] = 0; s.active[gi] = 1;
                s.a0[mfa] = (uint8_t)g; s.pr0[gi] = FREQ(g); s.pr1[gi] = 0.0;
                ++gi;
            }
            continue;
        }
        const int g1 = s.member[mfa], g2 = s.member[pfa];
        if (g1 != -1) {
            int f1 = s.fixed[g1];
            if (g2 != -1) {
                if (g1 == g2) {
                    if (f1 != -1) {
                        if (!fag_legal(g, ASG(s, f1, mfa), ASG(s, f1, pfa))) return 0.0;
                    } else {
                        const int l0 = fag_legal(g, s.a0[mfa], s.a0[pfa]);
                        const int l1 = fag_legal(g, s.a1[mfa], s.a1[pfa]);
                        if (l0) {
                            if (!l1) { s.fixed[g1] = 0; s.pr1[g1] = 0.0; }
                        } else {
                            if (l1) { s.fixed[g1] = 1; s.pr0[g1] = 0.0; }
                            else return 0.0;
                        }
                    }
                } else {
                    int f2 = s.fixed[g2];
                    if (f1 != -1) {
                        if (f2 != -1) {
                            if (!fag_legal(g, ASG(s, f1, mfa), ASG(s, f2, pfa))) return 0.0;
                        } else {
                            const int l0 = fag_legal(g, ASG(s, f1, mfa), s.a0[pfa]);
                            const int l1 = fag_legal(g, ASG(s, f1, mfa), s.a1[pfa]);
                            if (l0) f2 = 0; else if (l1) f2 = 1; else return 0.0;
                        }
                    } else if (f2 != -1) {
                        const int l0 = fag_legal(g, s.a0[mfa], ASG(s, f2, pfa));
                        const int l1 = fag_legal(g, s.a1[mfa], ASG(s, f2, pfa));
                        if (l0) f1 = 0; else if (l1) f1 = 1; else return 0.0;
                    } else {
                        const int l0 = fag_legal(g, s.a0[mfa], s.a0[pfa]);
                        const int l1 = fag_legal(g, s.a1[mfa], s.a0[pfa]);
                        const int l2 = fag_legal(g, s.a0[mfa], s.a1[pfa]);
                        const int l3 = fag_legal(g, s.a1[mfa], s.a1[pfa]);
                        if (!(l0 || l1 || l2 || l3)) return 0.0;
                        if (l0 && !(l1 || l2 || l3)) { f1 = 0; f2 = 0; }
                        else if (l1 && !(l0 || l2 || l3)) { f1 = 1; f2 = 0; }
                        else if (l2 && !(l0 || l1 || l3)) { f1 = 0; f2 = 1; }
                        else if (l3 && !(l0 || l1 || l2)) { f1 = 1; f2 = 1; }
                        else if (l0 && l3 && !(l1 || l2)) { f1 = -1; f2 = -1; }
                        else if (l1 && l2 && !(l0 || l3)) { f1 = -2; f2 = -2; }
                        else { f1 = -1; f2 = -1; }
                    }
                    if (f1 != f2) {
                        s.fixed[g1] = (int8_t)f1;
                        PRB(s, 1 - f1, g1) = 0.0;
                        PRB(s, 1 - f2, g2) = 0.0;
                        fag_combine(s, nfa, g1, g2, true);
                    } else if (f1 == -2) {
                        s.fixed[g1] = -1;
                        fag_combine(s, nfa, g1, g2, true);
                    } else {
                        s.fixed[g1] = (int8_t)f1;
                        if (f1 != -1) {
                            PRB(s, 1 - f1, g1) = 0.0;
                            PRB(s, 1 - f2, g2) = 0.0;
                        }
                        fag_combine(s, nfa, g1, g2, false);
                    }
                }
            } else {
                if (f1 != -1) {
                    const int t0 = fag_other(g, ASG(s, f1, mfa));
                    if (t0 == G_UNTYPED) return 0.0;
                    if (f1 == 0) s.a0[pfa] = (uint8_t)t0; else s.a1[pfa] = (uint8_t)t0;
                    PRB(s, f1, g1) = DMUL(PRB(s, f1, g1), FREQ(t0));
                } else {
                    const int t0 = fag_other(g, s.a0[mfa]);
                    const int t1 = fag_other(g, s.a1[mfa]);
                    if (t0 != G_UNTYPED) {
                        if (t1 != G_UNTYPED) {
                            s.a0[pfa] = (uint8_t)t0; s.a1[pfa] = (uint8_t)t1;
                            s.pr0[g1] = DMUL(s.pr0[g1], FREQ(t0));
                            s.pr1[g1] = DMUL(s.pr1[g1], FREQ(t1));
                        } else {
                            s.a0[pfa] = (uint8_t)t0;
                            s.pr0[g1] = DMUL(s.pr0[g1], FREQ(t0));
                            s.pr1[g1] = 0.0;
                            s.fixed[g1] = 0;
                        }
                    } else {
                        if (t1 != G_UNTYPED) {
                            s.a1[pfa] = (uint8_t)t1;
                            s.pr1[g1] = DMUL(s.pr1[g1], FREQ(t1));
                            s.pr0[g1] = 0.0;
                            s.fixed[g1] = 1;
                        } else return 0.0;
                    }
                }
                s.member[pfa] = (int16_t)g1;
            }
        } else if (g2 != -1) {
            const int f2 = s.fixed[g2];
            if (f2 != -1) {
                const int t0 = fag_other(g, ASG(s, f2, pfa));
                if (t0 == G_UNTYPED) return 0.0;
                if (f2 == 0) s.a0[mfa] = (uint8_t)t0; else s.a1[mfa] = (uint8_t)t0;
                PRB(s, f2, g2) = DMUL(PRB(s, f2, g2), FREQ(t0));
            } else {
                const int t0 = fag_other(g, s.a0[pfa]);
                const int t1 = fag_other(g, s.a1[pfa]);
                if (t0 != G_UNTYPED) {
                    if (t1 != G_UNTYPED) {
                        s.a0[mfa] = (uint8_t)t0; s.a1[mfa] = (uint8_t)t1;
                        s.pr0[g2] = DMUL(s.pr0[g2], FREQ(t0));
                        s.pr1[g2] = DMUL(s.pr1[g2], FREQ(t1));
                    } else {
                        s.a0[mfa] = (uint8_t)t0;
                        s.pr0[g2] = DMUL(s.pr0[g2], FREQ(t0));
                        s.pr1[g2] = 0.0;
                        s.fixed[g2] = 0;
                    }
                } else {
                    if (t1 != G_UNTYPED) {
                        s.a1[mfa] = (uint8_t)t1;
                        s.pr1[g2] = DMUL(s.pr1[g2], FREQ(t1));
                        s.pr0[g2] = 0.0;
                        s.fixed[g2] = 1;
                    } else return 0.0;
                }
            }
            s.member[mfa] = (int16_t)g2;
        } else {
            if (g == G_HETERO) {
                s.a0[mfa] = G_HOMOZ_A; s.a1[pfa] = G_HOMOZ_A;
                s.a1[mfa] = G_HOMOZ_B; s.a0[pfa] = G_HOMOZ_B;
                s.pr0[gi] = DMUL(major, minor);
                s.pr1[gi] = DMUL(major, minor);
                s.fixed[gi] = -1;
            } else {
                s.a0[mfa] = (uint8_t)g; s.a0[pfa] = (uint8_t)g;
                s.pr0[gi] = DMUL(FREQ(g), FREQ(g));
                s.pr1[gi] = 0.0;
                s.fixed[gi] = 0;
            }
            s.member[mfa] = (int16_t)gi;
            s.member[pfa] = (int16_t)gi;
            s.active[gi] = 1;
            ++gi;
        }
    }
#undef FREQ
    double ret = 1.0;
    for (int i = 0; i < gi; ++i) {
        if (!s.active[i]) continue;
        const int fx = s.fixed[i];
        if (fx != -1) ret = DMUL(ret, PRB(s, fx, i));
        else ret = DMUL(ret, DADD(s.pr0[i], s.pr1[i]));
    }
    return ret;
}

// ---------------------------------------------------------------------------
// M-sampler sweep: one block per chain.  Warp 0 runs the forward filter and
// backward sampling (serial along the map) with all 32 lanes computing the
// same recursion on values broadcast by shuffles from coalesced chunks.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) msampler_kernel(ProblemDev P, uint32_t* dg, int first, const int32_t* meioses,
                                                       int64_t meioses_chain_stride, int nm, Draws draws,
                                                       const uint8_t* sel, int want, double* rawbuf,
                                                       double* fbbuf, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int cr = blockIdx.x;
    if (sel && sel[cr] != want) return;
    const int chain = first + cr;
    const int tid = threadIdx.x, lane = tid & 31;
    FagState fs = fag_bind(smem + (size_t)tid * P.fag_bytes, P.N, P.F);
    uint32_t* G = dg + (size_t)chain * P.M * P.W;
    double* raw = rawbuf + (size_t)cr * 2 * P.M;
    double* fb = fbbuf + (size_t)cr * 2 * P.M;
    const int32_t* order = meioses + cr * meioses_chain_stride;
    __shared__ int bad;
    if (tid == 0) bad = 0;
    __syncthreads();
    // reset (meiosis_sampler.cc:17-40)
    const int m0 = order[0];
    for (int l = tid; l < P.M; l += blockDim.x) {
        const uint32_t* col = G + (size_t)l * P.W;
        fag_edges(P, col, fs, -1);
        const double lk = fag_like(P, l, fs);
        raw[2 * l + dgbit(col, m0)] = lk;
        if (lk == 0.0) bad = 1;
    }
    __syncthreads();
    if (bad) {
        if (tid == 0) set_status(status, ST_ILLEGAL_DG);
        return;
    }
    int last = m0;
    for (int j = 0; j < nm; ++j) {
        const int m = order[j];
        // likelihoods with meiosis m at both values (meiosis_sampler.cc:116-133)
        for (int l = tid; l < P.M; l += blockDim.x) {
            const uint32_t* col = G + (size_t)l * P.W;
            const int t = dgbit(col, m), t2 = dgbit(col, last);
            const double keep = raw[2 * l + t2];
            fag_edges(P, col, fs, m);
            const double lk = fag_like(P, l, fs);
            raw[2 * l + t] = keep;
            raw[2 * l + 1 - t] = lk;
            if (keep == 0.0 && lk == 0.0) bad = 1;
        }
        __syncthreads();
        if (bad) {
            if (tid == 0) set_status(status, ST_ILLEGAL_DG);
            return;
        }
        if (tid < 32) {
            // forward filter (meiosis_sampler.cc:136-155)
            double prev0 = 0.0, prev1 = 0.0;
            for (int base = 0; base < P.M; base += 32) {
                const int i = base + lane;
                const double r0 = i < P.M ? raw[2 * i] : 0.0;
                const double r1 = i < P.M ? raw[2 * i + 1] : 0.0;
                const double th = (i >= 1 && i < P.M) ? P.theta[i - 1] : 0.0;
                const int n = min(32, P.M - base);
                double k0 = 0.0, k1 = 0.0;
                for (int x = 0; x < n; ++x) {
                    const double a0 = __shfl_sync(FULLMASK, r0, x), a1 = __shfl_sync(FULLMASK, r1, x);
                    const double tx = __shfl_sync(FULLMASK, th, x);
                    double f0, f1;
                    if (base + x == 0) {
                        const double tot = DADD(a0, a1);
                        f0 = DDIV(a0, tot);
                        f1 = DDIV(a1, tot);
                    } else {
                        const double ax = DSUB(1.0, tx);
                        f0 = DMUL(a0, DADD(DMUL(prev1, tx), DMUL(prev0, ax)));
                        f1 = DMUL(a1, DADD(DMUL(prev0, tx), DMUL(prev1, ax)));
                        const double tt = DADD(f0, f1);
                        f0 = DDIV(f0, tt);
                        f1 = DDIV(f1, tt);
                    }
                    prev0 = f0;
                    prev1 = f1;
                    if (lane == x) { k0 = f0; k1 = f1; }
                }
                if (i < P.M) { fb[2 * i] = k0; fb[2 * i + 1] = k1; }
            }
            __syncwarp();
            // backward sampling (meiosis_sampler.cc:157-203)
            int64_t cursor = 0;
            int nxt = 0;
            for (int top = P.M - 1; top >= 0; top -= 32) {
                const int lo = max(0, top - 31);
                const int n = top - lo + 1;
                const int i = top - lane;
                const bool in = i >= lo;
                const double f0 = in ? fb[2 * i] : 0.0, f1 = in ? fb[2 * i + 1] : 0.0;
                const double th = (in && i < P.M - 1) ? P.theta[i] : 0.0;
                uint32_t* wp = in ? (G + (size_t)i * P.W + (m >> 5)) : nullptr;
                const int cur = in ? (int)((*wp >> (m & 31)) & 1u) : 0;
                const int64_t c0 = cursor;
                const double dr = (c0 + lane < P.M) ? draws.get(cr, chain, j, c0 + lane) : 0.0;
                int mine = cur;
                for (int x = 0; x < n; ++x) {
                    const int ii = top - x;
                    double a0 = __shfl_sync(FULLMASK, f0, x), a1 = __shfl_sync(FULLMASK, f1, x);
                    const double tx = __shfl_sync(FULLMASK, th, x);
                    if (ii < P.M - 1) {
                        const double ax = DSUB(1.0, tx);
                        a0 = DMUL(a0, nxt != 0 ? tx : ax);
                        a1 = DMUL(a1, nxt != 1 ? tx : ax);
                    }
                    int samp;
                    if (a0 == 0.0) samp = 1;
                    else if (a1 == 0.0) samp = 0;
                    else {
                        const double r = __shfl_sync(FULLMASK, dr, (int)(cursor - c0));
                        ++cursor;
                        samp = (r < DDIV(a0, DADD(a0, a1))) ? 0 : 1;
                    }
                    nxt = samp;
                    if (lane == x) mine = samp;
                }
                if (in && mine != cur) *wp ^= (1u << (m & 31));
            }
        }
        __syncthreads();
        last = m;
    }
}

// ---------------------------------------------------------------------------
// Trait peel LOD scorer: one warp per (graph, interval, position).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int phased_trait(int m, int p, int i, int j) {
    // rfunction.cc:98-114 with affected_trait (rfunction.h:82-107)
    const int ma = (m == AA) || (m == AU && i == 0) || (m == UA && i == 1);
    const int pa = (p == AA) || (p == AU && j == 0) || (p == UA && j == 1);
    if (ma) return pa ? AA : AU;
    return pa ? UA : UU;
}

template <typename T>
struct Arith;
template <>
struct Arith<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return DMUL(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return DADD(a, b); }
};
template <>
struct Arith<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
};

// TraitRfunction::get_recombination_probability (trait_rfunction.cc:9-24)
template <typename T>
__device__ __forceinline__ T trait_rec(int bits, int i, int j, T th, T an, T th2, T an2) {
    using Ar = Arith<T>;
    T tmp = ((bits & 1) == i) ? an : th;                      // maternal, locus
    tmp = Ar::mul(tmp, (((bits >> 2) & 1) == i) ? an2 : th2); // maternal, locus + 1
    tmp = Ar::mul(tmp, (((bits >> 1) & 1) == j) ? an : th);   // paternal, locus
    tmp = Ar::mul(tmp, (((bits >> 3) & 1) == j) ? an2 : th2); // paternal, locus + 1
    return tmp;
}

__device__ __forceinline__ int person_bits(const ProblemDev& P, const uint32_t* colL, const uint32_t* colR,
                                           int person) {
    const int b = 2 * (person - P.F);
    return dgbit(colL, b) | (dgbit(colL, b + 1) << 1) | (dgbit(colR, b) << 2) | (dgbit(colR, b + 1) << 3);
}

template <typename T, bool RESCALE>
__global__ void __launch_bounds__(128) lod_kernel(ProblemDev P, const uint32_t* graphs, int64_t graph_words,
                                                  int G, double* vals, int* status) {
    using Ar = Arith<T>;
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* A = (T*)(smem + (size_t)warp * P.arena * sizeof(T));
    const int n = P.n_lod;
    const int64_t npos = (int64_t)(P.M - 1) * n;
    const int64_t ntask = (int64_t)G * npos;
    for (int64_t t = (int64_t)blockIdx.x * wpb + warp; t < ntask; t += (int64_t)gridDim.x * wpb) {
        const int b = (int)(t / npos);
        const int64_t pidx = t % npos;
        const int l = (int)(pidx / n), o = (int)(pidx % n);
        const uint32_t* colL = graphs + (size_t)b * graph_words + (size_t)l * P.W;
        const uint32_t* colR = colL + P.W;
        // TraitRfunction::set_thetas (trait_rfunction.h:50-56)
        const double thd = DMUL(P.partial[l], (double)(o + 1));
        const double th2d = DMUL(P.partial[l], (double)(n + 1 - (o + 1)));
        const T th = (T)thd, an = (T)DSUB(1.0, thd), th2 = (T)th2d, an2 = (T)DSUB(1.0, th2d);
        const T quarter = (T)0.25;
        int scale = 0;
        for (int k = 0; k < P.K; ++k) {
            const OpDev op = P.ops[k];
            const int ncell = 1 << (2 * op.c);
            const int32_t* cut = P.opdata + op.cut_at;
            const double* trait = P.dprob + 4 * op.peel;
            T* out = A + op.mat_off;
            T mx = (T)0;
            for (int cell = lane; cell < ncell; cell += 32) {
                bool valid = true;
                for (int q = 0; q < op.c; ++q) valid &= ((P.dmask[cut[q]] >> digit(cell, q)) & 1) != 0;
                T total = (T)0;
                if (valid) {
                    if (op.type == CHILD) {
                        const int mt = digit(cell, op.mpos), pt = digit(cell, op.fpos);
                        const int bits = person_bits(P, colL, colR, op.peel);
                        for (int i = 0; i < 2; ++i)
                            for (int j = 0; j < 2; ++j) {
                                const int kt = phased_trait(mt, pt, i, j);
                                const double tvd = trait[kt];
                                if (tvd == 0.0) continue;
                                const int ext = cell | (kt << (2 * op.c));
                                T tmp = (T)tvd;
                                const int32_t* pd = P.opdata + op.prev_at;
                                for (int jj = 0; jj < op.n_prev; ++jj) {
                                    int idx = 0;
                                    for (int q = 0; q < pd[1]; ++q) idx |= digit(ext, pd[2 + q]) << (2 * q);
                                    tmp = Ar::mul(tmp, A[pd[0] + idx]);
                                    pd += 2 + pd[1];
                                }
                                tmp = Ar::mul(tmp, Ar::mul(quarter, trait_rec<T>(bits, i, j, th, an, th2, an2)));
                                total = Ar::add(total, tmp);
                            }
                    } else if (op.type == PARENT) {
                        for (int a = 0; a < 4; ++a) {
                            const double tvd = trait[a];
                            if (tvd == 0.0) continue;
                            const int ext = cell | (a << (2 * op.c));
                            T tmp = (T)tvd;
                            const int32_t* pd = P.opdata + op.prev_at;
                            for (int jj = 0; jj < op.n_prev; ++jj) {
                                int idx = 0;
                                for (int q = 0; q < pd[1]; ++q) idx |= digit(ext, pd[2 + q]) << (2 * q);
                                tmp = Ar::mul(tmp, A[pd[0] + idx]);
                                pd += 2 + pd[1];
                            }
                            T cp = (T)1;
                            int mt = a, pt = a;
                            const int32_t* cd = P.opdata + op.child_at;
                            for (int c = 0; c < op.n_child; ++c, cd += 4) {
                                const int kt = digit(ext, cd[1]), other = digit(ext, cd[2]);
                                if (cd[3]) pt = other; else mt = other;
                                const int bits = person_bits(P, colL, colR, cd[0]);
                                T ct = (T)0;
                                for (int i = 0; i < 2; ++i)
                                    for (int j = 0; j < 2; ++j) {
                                        if (phased_trait(mt, pt, i, j) != kt) continue;
                                        ct = Ar::add(ct, Ar::mul(quarter, trait_rec<T>(bits, i, j, th, an, th2, an2)));
                                    }
                                cp = Ar::mul(cp, ct);
                            }
                            tmp = Ar::mul(tmp, cp);
                            total = Ar::add(total, tmp);
                        }
                    } else {
                        for (int a = 0; a < 4; ++a) {
                            const double tvd = trait[a];
                            if (tvd == 0.0) continue;
                            const int ext = cell | (a << (2 * op.c));
                            T tmp = (T)tvd;
                            const int32_t* pd = P.opdata + op.prev_at;
                            for (int jj = 0; jj < op.n_prev; ++jj) {
                                int idx = 0;
                                for (int q = 0; q < pd[1]; ++q) idx |= digit(ext, pd[2 + q]) << (2 * q);
                                tmp = Ar::mul(tmp, A[pd[0] + idx]);
                                pd += 2 + pd[1];
                            }
                            total = Ar::add(total, tmp);
                        }
                    }
                }
                out[cell] = total;
                mx = total > mx ? total : mx;
            }
            __syncwarp();
            if (RESCALE) {
                for (int s = 16; s > 0; s >>= 1) {
                    const T o2 = __shfl_xor_sync(FULLMASK, mx, s);
                    mx = o2 > mx ? o2 : mx;
                }
                if (mx > (T)0) {
                    const int e = ilogbf((float)mx);
                    const T f = (T)scalbnf(1.0f, -e);
                    for (int cell = lane; cell < ncell; cell += 32) out[cell] *= f;
                    scale += e;
                }
                __syncwarp();
            }
        }
        if (lane == 0) {
            const double r = (double)A[P.ops[P.K - 1].mat_off];
            // DescentGraph::get_recombination_prob (descent_graph.cc:212-242)
            const double lt = log(P.theta[l]), la = log(DSUB(1.0, P.theta[l]));
            double rec = 0.0;
            for (int bb = 0; bb < 2 * P.Nnf; ++bb) rec = DADD(rec, dgbit(colL, bb) != dgbit(colR, bb) ? lt : la);
            double v;
            if (r <= 0.0) {
                set_status(status, ST_LOD_NONPOS);
                v = -DBL_MAX;
            } else {
                v = log(r) + (double)scale * 0.69314718055994530942 - rec - P.marker_trans;
            }
            vals[t] = v;
        }
        __syncwarp();
    }
}

// log_sum (logarithms.cc:14-25)
__device__ __forceinline__ double log_sum(double a, double b) {
    if (a == -DBL_MAX) return b;
    if (b == -DBL_MAX) return a;
    return log(exp(b - a) + 1.0) + a;
}

// LODscores::add in graph order (lod_score.h:74-80)
__global__ void lod_merge_kernel(const double* vals, int G, int64_t npos, double* acc, uint8_t* init) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npos; p += (int64_t)gridDim.x * blockDim.x) {
        double a = acc[p];
        uint8_t ini = init[p];
        for (int b = 0; b < G; ++b) {
            const double v = vals[(size_t)b * npos + p];
            a = ini ? log_sum(v, a) : v;
            ini = 1;
        }
        acc[p] = a;
        init[p] = ini;
    }
}

// Per-chain shuffled meiosis order for device-driven M-sweeps (the reference
// shuffles m_ordering each sweep, markov_chain.cc:346): Fisher-Yates with
// Philox draws.
__global__ void shuffle_kernel(const int32_t* base, int nm, int32_t* out, int first, int nchain, uint64_t seed,
                               uint64_t iter) {
    const int cr = blockIdx.x * blockDim.x + threadIdx.x;
    if (cr >= nchain) return;
    const int chain = first + cr;
    int32_t* o = out + (size_t)cr * nm;
    for (int i = 0; i < nm; ++i) o[i] = base[i];
    const uint64_t hi = ((uint64_t)chain << 40) ^ (iter << 4) ^ 3u;
    for (int i = nm - 1; i > 0; --i) {
        const double u = philox_u01(seed, hi, (uint64_t)i);
        int j = (int)(u * (double)(i + 1));
        if (j > i) j = i;
        const int32_t t = o[i];
        o[i] = o[j];
        o[j] = t;
    }
}

// One uniform per chain decides L- or M-sweep (markov_chain.cc:336-352).
__global__ void choose_kernel(int first, int nchain, uint64_t seed, uint64_t iter, double lprob, uint8_t* is_l) {
    const int cr = blockIdx.x * blockDim.x + threadIdx.x;
    if (cr >= nchain) return;
    const uint64_t hi = ((uint64_t)(first + cr) << 40) ^ (iter << 4) ^ 7u;
    is_l[cr] = philox_u01(seed, hi, 0) < lprob ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
size_t lsampler_smem_per_warp(const ProblemDev& P) {
    return (size_t)P.arena * 8 + (size_t)P.max_child * 128 + (((size_t)P.N + 15) & ~(size_t)15);
}

int fag_bytes(int N, int F) { return fag_state_bytes(N, F); }

cudaError_t launch_lsampler(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* loci, int nloci,
                            const double* u, int64_t ucs, int64_t uls, uint64_t seed, uint64_t iter,
                            const uint8_t* sel, int want, int* status, cudaStream_t s, int grid_cap, int wpb) {
    const size_t smem = wpb * lsampler_smem_per_warp(P);
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(lsampler_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    Draws d{u, ucs, uls, seed, iter, 1};
    const int64_t ntask = (int64_t)nchain * nloci;
    int64_t grid = (ntask + wpb - 1) / wpb;
    if (grid > grid_cap) grid = grid_cap;
    if (grid < 1) grid = 1;
    lsampler_kernel<<<(int)grid, wpb * 32, smem, s>>>(P, dg, first, nchain, loci, nloci, d, sel, want, status);
    return cudaGetLastError();
}

cudaError_t launch_msampler(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* meioses,
                            int64_t mstride, int nm, const double* u, int64_t ucs, uint64_t seed, uint64_t iter,
                            const uint8_t* sel, int want, double* raw, double* fb, int* status, int threads,
                            cudaStream_t s) {
    const size_t smem = (size_t)threads * P.fag_bytes;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(msampler_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    Draws d{u, ucs, P.M, seed, iter, 2};
    msampler_kernel<<<nchain, threads, smem, s>>>(P, dg, first, meioses, mstride, nm, d, sel, want, raw, fb, status);
    return cudaGetLastError();
}

cudaError_t launch_lod(const ProblemDev& P, int precision, const uint32_t* graphs, int64_t graph_words, int G,
                       double* vals, int* status, cudaStream_t s, int grid_cap, int wpb) {
    const int64_t ntask = (int64_t)G * (P.M - 1) * P.n_lod;
    int64_t grid = (ntask + wpb - 1) / wpb;
    if (grid > grid_cap) grid = grid_cap;
    if (grid < 1) grid = 1;
    if (precision == 0) {
        const size_t smem = (size_t)wpb * P.arena * sizeof(double);
        static size_t configured = 0;
        if (smem > configured) {
            cudaError_t e = cudaFuncSetAttribute(lod_kernel<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            configured = smem;
        }
        lod_kernel<double, false><<<(int)grid, wpb * 32, smem, s>>>(P, graphs, graph_words, G, vals, status);
    } else {
        const size_t smem = (size_t)wpb * P.arena * sizeof(float);
        static size_t configured = 0;
        if (smem > configured) {
            cudaError_t e = cudaFuncSetAttribute(lod_kernel<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            configured = smem;
        }
        lod_kernel<float, true><<<(int)grid, wpb * 32, smem, s>>>(P, graphs, graph_words, G, vals, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_lod_merge(const double* vals, int G, int64_t npos, double* acc, uint8_t* init, cudaStream_t s) {
    const int threads = 256;
    int64_t grid = (npos + threads - 1) / threads;
    if (grid > 65535) grid = 65535;
    lod_merge_kernel<<<(int)grid, threads, 0, s>>>(vals, G, npos, acc, init);
    return cudaGetLastError();
}

cudaError_t launch_shuffle(const int32_t* base, int nm, int32_t* out, int first, int nchain, uint64_t seed,
                           uint64_t iter, cudaStream_t s) {
    shuffle_kernel<<<(nchain + 63) / 64, 64, 0, s>>>(base, nm, out, first, nchain, seed, iter);
    return cudaGetLastError();
}

cudaError_t launch_choose(int first, int nchain, uint64_t seed, uint64_t iter, double lprob, uint8_t* is_l,
                          cudaStream_t s) {
    choose_kernel<<<(nchain + 63) / 64, 64, 0, s>>>(first, nchain, seed, iter, lprob, is_l);
    return cudaGetLastError();
}

}  // namespace sl
