// sm_103a kernels for the SwiftLink MCMC hot path.
//
// Samplers (one chain's descent graph per chain, bit-packed [chain][M][W]):
//  * lsampler_kernel<T,G> -- L-sampler, one group of G = 32, 16 or 8 lanes per
//                            (chain, locus): T=double with the reference's
//                            operation order (bit-exact decisions), T=float
//                            the batched form.  The form compiled per
//                            pedigree lives in sl_lsjit.cc.
//  * si_kernel<T>, si_select_kernel -- sequential imputation passes (one-sided
//                            L-steps from a start locus) and the best pass.
//  * fag_kernel           -- M-sampler likelihoods, thread per (chain, locus):
//                            founder-allele graph with one meiosis toggled
//                            (exact mode, and fast mode past the warp form's
//                            shared-memory limit).
//  * fag_warp_kernel<G>   -- the same in lane groups of G (fast mode).
//  * ffbs_kernel<T>       -- forward filter / backward sample of one meiosis,
//                            one warp per chain, in the reference's order.
//  * ffbs_scan_kernel     -- the same as block-wide scans (fast mode).
//  * loglik_*_kernel      -- log P(G, graph) of (graph, map) chain pairs (MC3).
// Scorer:
//  * lod_kernel<T,R>      -- trait peel at every (graph, interval, position), one
//                            warp per task; T=double is the plain FP64 form,
//                            R=true rescales every rfunction by a power of two
//                            and carries the exponent.
//  * lod_prog_kernel      -- the FP32 rescaled peel as a slot-program
//                            interpreter (specialised forms: sl_jit.cc).
//  * trait_adjoint_kernel, trait_adjoint_thr_kernel -- the hand-written
//                            adjoint of the rescaled peel, a warp or a thread
//                            per task (the form compiled per pedigree lives
//                            in sl_adjjit.cc).
//  * lod_merge_kernel, chain_merge_kernel -- FP64 log-sum accumulation.
// Run graph: run_init / chain_iter / chain_advance kernels drive each chain's
// WHILE and SWITCH nodes; choose / shuffle / set_key draw the iteration's
// choices; lfreq_kernel precomputes the allele frequencies' log2 per chain map.
//
// FP64 arithmetic on decision paths uses __dmul_rn/__dadd_rn/__ddiv_rn so no
// multiply-add is contracted and the doubles match the reference's.

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "sl_internal.h"
#include "sl_philox.cuh"

namespace sl {

// Raises a kernel's dynamic shared-memory limit on the current device when a
// launch needs more than it was given so far.  The attribute is per device
// and contexts on several devices or threads may launch the same kernel, so
// the record is keyed by (kernel, device) and taken under a lock.
static cudaError_t ensure_smem(const void* func, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> given;
    std::lock_guard<std::mutex> lock(mu);
    size_t& have = given[std::make_pair(func, dev)];
    if (bytes <= have) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) have = bytes;
    return e;
}

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

__device__ __forceinline__ double philox_u01(uint64_t key, uint64_t c_hi, uint64_t c_lo) {
    return sl_philox_u01(key, c_hi, c_lo);
}

// Where uniform draws come from: a caller-supplied array (bit-exact replay of
// the reference) or the Philox stream (device-driven runs).  `unit` is the
// locus (L-sampler) or the meiosis step (M-sampler) within the sweep.
// `key` (device memory, may be null) overrides seed and iteration: a
// captured graph replayed every iteration reads them there.
struct Draws {
    const double* u;
    int64_t chain_stride, unit_stride;
    uint64_t seed, iter;
    int stage;
    const uint64_t* key;
    __device__ __forceinline__ double get(int chain_rel, int chain, int64_t unit, int64_t k) const {
        if (u) return u[chain_rel * chain_stride + unit * unit_stride + k];
        const uint64_t sd = key ? key[0] : seed, it = key ? key[1] : iter;
        uint64_t hi = ((uint64_t)chain << 40) ^ (it << 4) ^ (uint64_t)stage;
        return philox_u01(sd, hi, ((uint64_t)unit << 24) ^ (uint64_t)k);
    }
};

__global__ void set_key_kernel(uint64_t* key, uint64_t seed, uint64_t iter) {
    key[0] = seed;
    key[1] = iter;
}

// Arithmetic of the L-sampler: FP64 without contraction (the reference's
// doubles) or plain FP32 for the fast sampler mode.
template <typename T>
struct Ls;
template <>
struct Ls<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return DMUL(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return DADD(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return DSUB(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return DDIV(a, b); }
};
template <>
struct Ls<float> {   // rounded operations, never contracted: the kernel specialised at run time matches them
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

// The lanes working on one L-sampler task: a whole warp (G = 32), half of one
// or a quarter (G = 16 or 8; two or four tasks per warp, for pedigrees whose
// rfunctions have few allowed cells).  Shuffles and ballots stay within the
// group, whose tasks may diverge from the warp's other groups; lane numbers
// are the group's own.
template <int G>
struct Lanes {
    static_assert(G == 32 || G == 16 || G == 8, "a lane group is 32, 16 or 8 lanes of one warp");
    unsigned mask;
    // the group's lanes: G consecutive lanes starting at a multiple of G
    __device__ __forceinline__ Lanes() : mask(G == 32 ? FULLMASK : (((1u << G) - 1u) << (threadIdx.x & (32 - G)))) {}
    template <typename V>
    __device__ __forceinline__ V shfl(V v, int src) const { return __shfl_sync(mask, v, src, G); }
    template <typename V>
    __device__ __forceinline__ V shfl_xor(V v, int d) const { return __shfl_xor_sync(mask, v, d, G); }
    template <typename V>
    __device__ __forceinline__ V shfl_up(V v, int d) const { return __shfl_up_sync(mask, v, d, G); }
    __device__ __forceinline__ unsigned ballot(bool p) const {
        const unsigned b = __ballot_sync(mask, p);
        return G == 32 ? b : (b >> (threadIdx.x & (32 - G))) & ((1u << G) - 1u);
    }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
};

// ---------------------------------------------------------------------------
// L-sampler
// ---------------------------------------------------------------------------

// Recombination distributions of one child's two meioses for every parental
// state (SamplerRfunction::get_recombination_distribution,
// sampler_rfunction.cc:102-157): d[side*8 + state*2 + allele].
template <typename T>
__device__ void ls_dist_one(const ProblemDev& P, int person, const uint32_t* colL, const uint32_t* colR,
                            int l, T th, T an, T th2, T an2, T* d) {
    using A = Ls<T>;
    for (int side = 0; side < 2; ++side) {
        const int b = 2 * (person - P.F) + side;
        T* s = d + side * 8;
        s[UU * 2 + 0] = T(1); s[UU * 2 + 1] = T(0);
        s[AA * 2 + 0] = T(0); s[AA * 2 + 1] = T(1);
        T tmp0 = T(0.5), tmp1 = T(0.5);
        if (colL) {   // a left neighbour (absent at locus 0 and when imputation ignores it)
            const bool cross = dgbit(colL, b) != 0;
            tmp0 = A::mul(tmp0, cross ? th2 : an2);
            tmp1 = A::mul(tmp1, cross ? an2 : th2);
        }
        if (colR) {
            const bool cross = dgbit(colR, b) != 0;
            tmp0 = A::mul(tmp0, cross ? th : an);
            tmp1 = A::mul(tmp1, cross ? an : th);
        }
        const T total = A::add(tmp0, tmp1);
        const T uau = A::div(tmp1, total);
        s[AU * 2 + 0] = uau;
        s[AU * 2 + 1] = A::sub(T(1), uau);
        const T uua = A::div(tmp0, total);
        s[UA * 2 + 0] = uua;
        s[UA * 2 + 1] = A::sub(T(1), uua);
    }
}

template <typename T, int G>
__device__ __forceinline__ void ls_dists(const ProblemDev& P, const OpDev& op, const int32_t* opd,
                                         const uint32_t* colL, const uint32_t* colR, int l, T th, T an, T th2, T an2,
                                         T* dist, int lane) {
    const int nch = op.type == CHILD ? 1 : (op.type == PARENT ? op.n_child : 0);
    for (int c = lane; c < nch; c += G) {
        const int person = op.type == CHILD ? op.peel : opd[op.child_at + 4 * c];
        ls_dist_one<T>(P, person, colL, colR, l, th, an, th2, an2, dist + 16 * c);
    }
}

// A cell of op k in the compact layout, with the peel node's state v: ext
// holds the dense digits of (cutset states, v) as in peel_matrix.h:37-45, rk
// the states' ranks and bits each position's rank bits (2 bits per position,
// the peel node at position c), bad the positions whose state is not allowed
// (only the peel node's can be, the cell itself being valid).
struct LsCell {
    int ext, rk, bits, bad;
};

// A task's compact rfunctions: the first `cap` cells in the task's shared
// memory, the rest (at the few loci whose rfunctions need more) in its slice
// of a global spill buffer.  Sizing the shared part for nearly every locus
// rather than the largest keeps more tasks resident on an SM.
template <typename T>
struct LsArena {
    T* sh;
    T* gl;
    int cap;
    __device__ __forceinline__ T ld(int o) const { return o < cap ? sh[o] : gl[o - cap]; }
    __device__ __forceinline__ void st(int o, T v) const {
        if (o < cap) sh[o] = v;
        else gl[o - cap] = v;
    }
};

// One presum entry (cell, peel state v) in the reference's product order
// (sampler_rfunction.cc:190-287, rfunction.cc:116-142); a previous rfunction
// is read at its compact index, or as zero where the dense matrix held zero.
template <typename T>
__device__ T ls_term(const OpDev& op, const int32_t* opd, const LsArena<T>& Am, const uint16_t* off, const T* dist,
                     const LsCell& x, int v, T tv) {
    using A = Ls<T>;
    const int ext = x.ext;
    T tmp = tv;
    if (op.type == CHILD) {
        const int mt = digit(ext, op.mpos), pt = digit(ext, op.fpos);
        const T tr = A::mul(dist[mt * 2 + mat_allele(v)], dist[8 + pt * 2 + pat_allele(v)]);
        tmp = A::mul(tmp, tr);
    }
    const int32_t* pd = opd + op.prev_at;
    const int32_t* po = opd + op.prev_ops_at;
    for (int j = 0; j < op.n_prev; ++j) {
        const int pc = pd[1];
        int idx = 0, sh = 0, bad = 0;
        for (int q = 0; q < pc; ++q) {
            const int pos = pd[2 + q];
            idx |= ((x.rk >> (2 * pos)) & 3) << sh;
            sh += (x.bits >> (2 * pos)) & 3;
            bad |= (x.bad >> pos) & 1;
        }
        tmp = A::mul(tmp, bad ? T(0) : Am.ld(off[po[j]] + idx));
        pd += 2 + pc;
    }
    if (op.type == PARENT) {
        T cp = T(1);
        const int32_t* cd = opd + op.child_at;
        for (int c = 0; c < op.n_child; ++c, cd += 4) {
            const int kt = digit(ext, cd[1]), other = digit(ext, cd[2]);
            const int mt = cd[3] ? v : other, pt = cd[3] ? other : v;
            const T tr = A::mul(dist[c * 16 + mt * 2 + mat_allele(kt)], dist[c * 16 + 8 + pt * 2 + pat_allele(kt)]);
            cp = A::mul(cp, tr);
        }
        tmp = A::mul(tmp, cp);
    }
    return tmp;
}

// The L-sampler's compact rfunctions.  At locus l a member whose genotype-
// elimination mask allows s states takes b = 0, 1 or 2 bits (s = 1, 2, 3-4)
// of a cell's index, holding the rank of its state among the allowed ones, in
// cutset order; op k's cells are the 2^B_k indices (B_k the sum of its
// members' bits) at offset off[k] of the task's arena, a prefix sum over the
// ops worked out at the start of each task.  Only cells whose members are all
// in allowed states are stored -- on the 400-member pedigree at most 1,350
// values against 11,485 for dense 4^c matrices -- and exactly those are the
// cells the dense layout could hold non-zero: a gather that would reach a
// dense cell with a disallowed state reads zero instead, and a rank past the
// allowed count (s = 3) marks an invalid cell.
__device__ __forceinline__ int rank_bits(int mask) {
    const int s = __popc(mask);
    return s <= 1 ? 0 : (s == 2 ? 1 : 2);
}
__device__ __forceinline__ int state_rank(int mask, int v) { return __popc(mask & ((1 << v) - 1)); }
__device__ __forceinline__ int state_of_rank(int mask, int r) {   // the r-th allowed state (r < popc(mask))
    for (int i = 0; i < r; ++i) mask &= mask - 1;
    return __ffs(mask) - 1;
}

// A task's shared bytes: the rfunctions [ls_arena, compact], the children's
// transmission distributions [16 per child], the sampled states [N], the
// locus's genotype codes and masks [N], its neighbours' descent-graph words
// [2 W], its prior row [16] and the ops' compact offsets [K + 1] (16-bit); each part
// 16-byte aligned, so every task's base is aligned.  (The backward pass's
// draws are made as it goes, one per operation: storing them took K doubles,
// a third of a task on the 400-member pedigree.)
__host__ __device__ __forceinline__ size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }
template <typename T>
__host__ __device__ __forceinline__ size_t ls_draws_at(const ProblemDev& P) {
    return al16((size_t)P.ls_cap * sizeof(T) + (size_t)P.max_child * 16 * sizeof(T) + (size_t)P.N);
}
template <typename T>
__host__ __device__ __forceinline__ size_t ls_gcol_at(const ProblemDev& P) {
    return ls_draws_at<T>(P);
}
template <typename T>
__host__ __device__ __forceinline__ size_t ls_cols_at(const ProblemDev& P) {
    return al16(ls_gcol_at<T>(P) + (size_t)P.N);
}
template <typename T>
__host__ __device__ __forceinline__ size_t ls_pri_at(const ProblemDev& P) {
    return al16(ls_cols_at<T>(P) + 8 * (size_t)P.W);
}
template <typename T>
__host__ __device__ __forceinline__ size_t ls_off_at(const ProblemDev& P) {
    return al16(ls_pri_at<T>(P) + 16 * sizeof(T));
}
template <typename T>
__host__ __device__ __forceinline__ size_t ls_warp_bytes(const ProblemDev& P) {
    return al16(ls_off_at<T>(P) + 2 * ((size_t)P.K + 1));   // 16-bit offsets: the arena holds < 65,536 cells
}

// Task slot s's part of the spill buffer of chain `chain` (null when no
// locus spills, or past the buffer's slots).  Every chain has its own slots:
// the run graph launches the chains' sweeps concurrently; a launch over
// several chains runs its tasks slot by slot in the first chain's slots.
template <typename T>
__device__ __forceinline__ T* ls_spill_slice(const ProblemDev& P, int chain, int64_t s) {
    if (P.ls_spill_cells <= 0 || s >= P.ls_spill_slots || chain < 0 || chain >= P.ls_spill_chains) return nullptr;
    return (T*)P.ls_spill + ((size_t)chain * P.ls_spill_slots + s) * P.ls_spill_cells;
}

// Block-shared copies of the peel's operations and their lists: every lane
// reads them at every operation, and L1 holds little beside the arenas.
__host__ __device__ __forceinline__ size_t ls_tables_bytes(const ProblemDev& P) {
    return P.ls_stage_ops ? al16((size_t)P.K * sizeof(OpDev)) + al16((size_t)P.opdata_n * 4) : 0;
}

__device__ __forceinline__ void ls_stage_tables(const ProblemDev& P, unsigned char* smem, const OpDev*& ops,
                                                const int32_t*& opd) {
    if (!P.ls_stage_ops) {   // tables too large to share a block's shared memory with the arenas
        ops = P.ops;
        opd = P.opdata;
        return;
    }
    int32_t* so = (int32_t*)smem;
    int32_t* sd = (int32_t*)(smem + al16((size_t)P.K * sizeof(OpDev)));
    const int32_t* src = (const int32_t*)P.ops;
    const int nw = P.K * (int)(sizeof(OpDev) / 4);
    for (int i = threadIdx.x; i < nw; i += blockDim.x) so[i] = src[i];
    for (int i = threadIdx.x; i < P.opdata_n; i += blockDim.x) sd[i] = P.opdata[i];
    ops = (const OpDev*)so;
    opd = sd;
}

// One warp per (chain, locus) task; the listed loci must be pairwise
// non-adjacent so each task owns its descent-graph column.
// One L-sampler step at locus l of one chain, by one warp
// (LocusSampler::step, locus_sampler2.cc:128-159): hasL / hasR say whether the
// neighbouring columns take part (set_locus(l, ignore_left, ignore_right),
// sampler_rfunction.h:84-101).  Draws are taken at indices base, base + 1, ...
// of the unit's stream.  Returns the number of draws used, or -1 when the
// locus has likelihood 0; *logroot (lane 0) receives log of the peel's result.
template <typename T, int G>
__device__ int ls_locus(const ProblemDev& P, const OpDev* ops, const int32_t* opd, uint32_t* dg, int cr, int chain,
                        int l, bool hasL, bool hasR, const Draws& draws, int64_t unit, int64_t base,
                        unsigned char* wsmem, T* spill, int lane, int* status, double* logroot) {
    using Ar = Ls<T>;
    const Lanes<G> L;
    constexpr bool kRescale = sizeof(T) == 4;   // FP32: each rfunction scaled to a maximum of about 1
    const LsArena<T> A{(T*)wsmem, spill, P.ls_cap};
    T* dist = A.sh + P.ls_cap;
    int8_t* assign = (int8_t*)(dist + 16 * P.max_child);
    uint16_t* off = (uint16_t*)(wsmem + ls_off_at<T>(P));
    uint32_t* colC = dg + ((size_t)chain * P.M + l) * P.W;
    // the locus's inputs copied to the task's shared memory first
    uint8_t* sg = (uint8_t*)(wsmem + ls_gcol_at<T>(P));
    uint32_t* sL = (uint32_t*)(wsmem + ls_cols_at<T>(P));
    uint32_t* sR = sL + P.W;
    T* spri = (T*)(wsmem + ls_pri_at<T>(P));
    {
        const uint8_t* gsrc = P.geno + (size_t)l * P.N;
        for (int i = lane; i < P.N; i += G) sg[i] = gsrc[i];
        for (int w = lane; w < P.W; w += G) {
            if (hasL) sL[w] = colC[w - P.W];
            if (hasR) sR[w] = colC[w + P.W];
        }
        for (int i = lane; i < 16; i += G) {
            if constexpr (sizeof(T) == 4) spri[i] = (T)P.prior_f[(size_t)l * 16 + i];
            else spri[i] = (T)P.prior[(size_t)l * 16 + i];
        }
        L.sync();
    }
    const uint32_t* colL = hasL ? sL : nullptr;
    const uint32_t* colR = hasR ? sR : nullptr;
    T th = T(1), an = T(1), th2 = T(1), an2 = T(1);
    if constexpr (sizeof(T) == 4) {
        const float* tf = P.c_theta_f + (size_t)chain * (P.M - 1);
        if (hasL) { th2 = tf[l - 1]; an2 = 1.f - th2; }
        if (hasR) { th = tf[l]; an = 1.f - th; }
    } else {
        const double* td = P.c_theta + (size_t)chain * (P.M - 1);
        if (hasL) { th2 = td[l - 1]; an2 = DSUB(1.0, td[l - 1]); }
        if (hasR) { th = td[l]; an = DSUB(1.0, td[l]); }
    }
    const uint8_t* gcol = sg;
    const T* pri = spri;
    int scale = 0;
    // the ops' compact offsets at this locus: each lane sums the cells of a
    // run of ops, a scan over the group turns the sums into offsets
    {
        const int per = (P.K + G - 1) / G, k0 = min(P.K, lane * per), k1 = min(P.K, k0 + per);
        int sum = 0;
        for (int k = k0; k < k1; ++k) {
            const OpDev& op = ops[k];
            int b = 0;
            for (int q = 0; q < op.c; ++q) b += rank_bits((gcol[opd[op.cut_at + q]] >> 4) & 15);
            sum += 1 << b;
        }
        int incl = sum;
        for (int dd = 1; dd < G; dd <<= 1) {
            const int o = L.shfl_up(incl, dd);
            if (lane >= dd) incl += o;
        }
        int run = incl - sum;
        for (int k = k0; k < k1; ++k) {
            const OpDev& op = ops[k];
            int b = 0;
            for (int q = 0; q < op.c; ++q) b += rank_bits((gcol[opd[op.cut_at + q]] >> 4) & 15);
            off[k] = (uint16_t)run;
            run += 1 << b;
        }
        if (lane == G - 1) off[P.K] = (uint16_t)incl;
        L.sync();
        if (L.shfl(incl, G - 1) > P.ls_arena || (spill == nullptr && L.shfl(incl, G - 1) > P.ls_cap)) {
            // cannot happen: the arena (shared part and spill) holds the most any locus needs
            if (lane == 0) set_status(status, ST_ILLEGAL_DG);
            return -1;
        }
    }
    // forward peel over the valid cells of every rfunction
    for (int k = 0; k < P.K; ++k) {
        const OpDev op = ops[k];
        ls_dists<T, G>(P, op, opd, colL, colR, l, th, an, th2, an2, dist, lane);
        L.sync();
        const int32_t* cut = opd + op.cut_at;
        // the op's members: allowed states (4 bits each) and rank bits, the peel node last
        unsigned long long mk = 0;
        int bits = 0, B = 0;
        for (int q = 0; q < op.c; ++q) {
            const int m = (gcol[cut[q]] >> 4) & 15, b = rank_bits(m);
            mk |= (unsigned long long)m << (4 * q);
            bits |= b << (2 * q);
            B += b;
        }
        const int mp = (gcol[op.peel] >> 4) & 15;
        bits |= rank_bits(mp) << (2 * op.c);
        const int ncell = 1 << B;
        const T* trait = pri + 4 * (gcol[op.peel] & 3);
        const int ob = off[k];
        T mx = T(0);
        // one (cell, state) term per lane, four lanes per cell; the cell's
        // total adds its terms in state order from zero, as the reference's
        // loop does (a skipped term is an exact zero)
        const int nitem = 4 * ncell, grp = lane & ~3, v = lane & 3;
        const T tv = trait[v];
        LsCell x;
        x.bits = bits;
        x.bad = ((mp >> v) & 1) ? 0 : 1 << op.c;
        const int vrank = state_rank(mp, v);
        for (int it0 = 0; it0 < nitem; it0 += G) {
            const int cell = (it0 + lane) >> 2;
            T term = T(0);
            if (it0 + lane < nitem && tv != T(0)) {
                // decode the compact index into states and ranks
                int rem = cell, ext = 0, rk = 0;
                bool ok = true;
                for (int q = 0; q < op.c; ++q) {
                    const int m = (int)(mk >> (4 * q)) & 15, b = (bits >> (2 * q)) & 3;
                    const int r = rem & ((1 << b) - 1);
                    rem >>= b;
                    ok &= r < __popc(m);
                    ext |= state_of_rank(m, r & 3) << (2 * q);
                    rk |= r << (2 * q);
                }
                if (ok) {
                    x.ext = ext | (v << (2 * op.c));
                    x.rk = rk | (vrank << (2 * op.c));
                    term = ls_term<T>(op, opd, A, off, dist, x, v, tv);
                }
            }
            const T t0 = L.shfl(term, grp), t1 = L.shfl(term, grp + 1);
            const T t2 = L.shfl(term, grp + 2), t3 = L.shfl(term, grp + 3);
            if (v == 0 && it0 + lane < nitem) {
                const T total = Ar::add(Ar::add(Ar::add(Ar::add(T(0), t0), t1), t2), t3);
                A.st(ob + cell, total);
                mx = total > mx ? total : mx;
            }
        }
        if (kRescale) {
            // the sampling draws from ratios within one rfunction, so a
            // power-of-two factor per rfunction changes no decision
            for (int dd = G / 2; dd >= 1; dd >>= 1) {
                const T o = L.shfl_xor(mx, dd);
                mx = o > mx ? o : mx;
            }
            if (mx > T(0)) {
                // every rfunction enters the root exactly once, so the root's
                // logarithm is the scaled root's plus the removed exponents
                const int ex = ilogbf((float)mx);
                scale += ex;
                const float f = scalbnf(1.0f, -ex);
                L.sync();   // the cells other lanes of the group wrote (some maybe in the global spill)
                for (int cell = lane; cell < ncell; cell += G) A.st(ob + cell, (T)((float)A.ld(ob + cell) * f));
            }
        }
        L.sync();
    }
    const T root = A.ld(off[P.K - 1]);
    if (root == T(0)) {
        if (lane == 0) set_status(status, ST_ZERO_LIK);
        L.sync();
        return -1;
    }
    if (lane == 0 && logroot) *logroot = log((double)root) + (double)scale * 0.69314718055994530942;
    for (int i = lane; i < P.N; i += G) assign[i] = -1;
    L.sync();
    // backward sampling of ordered genotypes (SamplerRfunction::sample); the
    // group's last lane draws the operation's uniform (one per operation, in
    // the backward order) while the others work out its terms
    for (int k = P.K - 1; k >= 0; --k) {
        const OpDev op = ops[k];
        const double rdraw = lane == G - 1 ? draws.get(cr, chain, unit, base + (P.K - 1 - k)) : 0.0;
        ls_dists<T, G>(P, op, opd, colL, colR, l, th, an, th2, an2, dist, lane);
        L.sync();
        const int32_t* cut = opd + op.cut_at;
        const T* trait = pri + 4 * (gcol[op.peel] & 3);
        // the sampled cutset states as a compact cell (invalid where a state
        // is not allowed: the dense matrix held zero there)
        int ext = 0, rk = 0, bits = 0;
        bool known = true, ok = true;
        for (int q = 0; q < op.c; ++q) {
            const int a = assign[cut[q]];
            const int m = (gcol[cut[q]] >> 4) & 15;
            known &= a >= 0;
            ok &= ((m >> (a & 3)) & 1) != 0;
            ext |= (a & 3) << (2 * q);
            rk |= state_rank(m, a & 3) << (2 * q);
            bits |= rank_bits(m) << (2 * q);
        }
        const int mp = (gcol[op.peel] >> 4) & 15;
        T pv = T(0);
        if (lane < 4 && known && ok) {
            const T tv = trait[lane];
            if (tv != T(0)) {
                LsCell x;
                x.ext = ext | (lane << (2 * op.c));
                x.rk = rk | (state_rank(mp, lane) << (2 * op.c));
                x.bits = bits | (rank_bits(mp) << (2 * op.c));
                x.bad = ((mp >> lane) & 1) ? 0 : 1 << op.c;
                pv = ls_term<T>(op, opd, A, off, dist, x, lane, tv);
            }
        }
        const double rk_draw = L.shfl(rdraw, G - 1);
        const T p0 = L.shfl(pv, 0), p1 = L.shfl(pv, 1);
        const T p2 = L.shfl(pv, 2), p3 = L.shfl(pv, 3);
        if (lane == 0) {
            if (!known) set_status(status, ST_ILLEGAL_DG);
            T pd[4] = {p0, p1, p2, p3};
            const T tot = Ar::add(Ar::add(Ar::add(p0, p1), p2), p3);
            if (tot != T(0))
                for (int v = 0; v < 4; ++v) pd[v] = Ar::div(pd[v], tot);
            const double r = rk_draw;
            T acc = T(0);
            int lastv = 0, pick = -1;
            for (int v = 0; v < 4; ++v) {
                acc = Ar::add(acc, pd[v]);
                if (r < (double)acc) { pick = v; break; }
                if (pd[v] != T(0)) lastv = v;
            }
            assign[op.peel] = (int8_t)(pick >= 0 ? pick : lastv);
        }
        L.sync();
    }
    // meiosis indicators (locus_sampler2.cc:32-125) in person order, maternal
    // first: bit b = 2 (person - F) + parent, so 32 consecutive meioses are one
    // descent-graph word.  A lane takes one meiosis; a draw is consumed only
    // below a homozygous parent, and a ballot prefix gives each draw its index.
    {
        int64_t cursor = base + P.K;
        const int nb = 2 * P.Nnf;
        for (int w = 0; w < P.W; ++w) {
            uint32_t word = 0;
            for (int h = 0; h < 32; h += G) {
                const int b = 32 * w + h + lane;
                int mi = 0, need = 0;
                T p0 = T(1), p1 = T(1);
                if (b < nb) {
                    const int i = P.F + (b >> 1), par = b & 1;
                    const int tr = assign[i];
                    const int ptr = assign[par == 0 ? P.mother[i] : P.father[i]];
                    const int allele = par == 0 ? ((tr == UU || tr == UA) ? 0 : 1) : ((tr == UU || tr == AU) ? 0 : 1);
                    if (ptr == UA || ptr == AU) {
                        mi = allele == 0 ? (ptr == UA ? 0 : 1) : (ptr == UA ? 1 : 0);
                    } else {
                        need = 1;
                        if (hasL) {
                            const int d = dgbit(colL, b);
                            p0 = Ar::mul(p0, d == 0 ? an2 : th2);
                            p1 = Ar::mul(p1, d == 1 ? an2 : th2);
                        }
                        if (hasR) {
                            const int d = dgbit(colR, b);
                            p0 = Ar::mul(p0, d == 0 ? an : th);
                            p1 = Ar::mul(p1, d == 1 ? an : th);
                        }
                    }
                }
                const unsigned nmask = L.ballot(need);
                if (need) {
                    const double r = draws.get(cr, chain, unit, cursor + __popc(nmask & ((1u << lane) - 1u)));
                    mi = (r < (double)Ar::div(p0, Ar::add(p0, p1))) ? 0 : 1;
                }
                cursor += __popc(nmask);
                word |= L.ballot(mi != 0) << h;
            }
            if (lane == 0) colC[w] = word;   // bits past 2 Nnf stay zero
        }
        L.sync();
        return (int)(cursor - base);
    }
}

// One task per (chain, locus), G lanes each (a warp, or half of one); the
// listed loci must be pairwise non-adjacent so each task owns its
// descent-graph column.
template <typename T, int G>
__global__ void __launch_bounds__(128) lsampler_kernel(ProblemDev P, uint32_t* dg, int first, int nchain,
                                                       const int32_t* loci, int nloci, Draws draws,
                                                       const uint8_t* sel, int want, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int kPer = 32 / G;   // tasks per warp
    const int tpb = (blockDim.x >> 5) * kPer, slot = (threadIdx.x >> 5) * kPer + ((threadIdx.x & 31) / G);
    const int lane = threadIdx.x & (G - 1);
    const OpDev* ops;
    const int32_t* opd;
    ls_stage_tables(P, smem, ops, opd);
    __syncthreads();
    unsigned char* wsmem = smem + ls_tables_bytes(P) + (size_t)slot * ls_warp_bytes<T>(P);
    T* spill = ls_spill_slice<T>(P, first, (int64_t)blockIdx.x * tpb + slot);
    if (P.ls_spill_cells > 0 && !spill) {   // the launch has more task slots than the spill buffer: never run past it
        if (lane == 0) set_status(status, ST_ILLEGAL_DG);
        return;
    }
    const int64_t ntask = (int64_t)nchain * nloci;
    for (int64_t t = (int64_t)blockIdx.x * tpb + slot; t < ntask; t += (int64_t)gridDim.x * tpb) {
        const int cr = (int)(t / nloci);
        if (sel && sel[cr] != want) continue;
        const int l = loci[t % nloci];
        ls_locus<T, G>(P, ops, opd, dg, cr, first + cr, l, l > 0, l < P.M - 1, draws, l, 0, wsmem, spill, lane,
                       status, nullptr);
    }
}

// Sequential imputation (LocusSampler::start_from, locus_sampler2.cc:214-241),
// one warp per chain: the start locus with neither neighbour, then leftwards
// with the right neighbour only, then rightwards with the left neighbour only;
// draws are consumed in one sequence (unit `unit`), the weight is the sum of
// log(root) over the steps (-DBL_MAX when a locus has likelihood 0).
// npass independent passes of every chain run as separate warps: pass q of
// chain cr writes the graph set at dg + q * pass_stride, draws from the
// Philox stream of pass draws.iter + q, starts at starts[q * nchain + cr] and
// leaves its weight at weights[q * nchain + cr].
template <typename T>
__global__ void __launch_bounds__(128) si_kernel(ProblemDev P, uint32_t* dg, int first, int nchain,
                                                 const int32_t* starts, Draws draws, int64_t unit, double* weights,
                                                 int* status, int npass, int64_t pass_stride) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const OpDev* ops;
    const int32_t* opd;
    ls_stage_tables(P, smem, ops, opd);
    __syncthreads();
    unsigned char* wsmem = smem + ls_tables_bytes(P) + (size_t)warp * ls_warp_bytes<T>(P);
    T* spill = ls_spill_slice<T>(P, first, (int64_t)blockIdx.x * wpb + warp);
    if (P.ls_spill_cells > 0 && !spill) {
        if (lane == 0) set_status(status, ST_ILLEGAL_DG);
        return;
    }
    for (int t = blockIdx.x * wpb + warp; t < nchain * npass; t += gridDim.x * wpb) {
        const int cr = t % nchain, q = t / nchain;
        const int chain = first + cr, M = P.M, start = starts[t];
        uint32_t* dgq = dg + (size_t)q * pass_stride;
        Draws dq = draws;
        dq.iter = draws.iter + (uint64_t)q;
        int64_t base = 0;
        double w = 0.0;
        bool ok = true;
        for (int v = 0; v < M && ok; ++v) {
            const int l = v == 0 ? start : (v <= start ? start - v : v);
            const bool hasL = v > start && l > 0;
            const bool hasR = v > 0 && v <= start && l < M - 1;
            double lr = 0.0;
            const int used = ls_locus<T, 32>(P, ops, opd, dgq, cr, chain, l, hasL, hasR, dq, unit, base, wsmem,
                                             spill, lane, status, &lr);
            if (used < 0) {
                ok = false;
                break;
            }
            base += used;
            w += __shfl_sync(FULLMASK, lr, 0);
        }
        if (lane == 0) weights[t] = ok ? w : -DBL_MAX;
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Founder allele graph likelihood (FounderAlleleGraph4::likelihood,
// founder_allele_graph4.cc:34-442), one thread per (chain, locus).  The
// per-thread state lives in shared memory as structure-of-arrays over the
// block's threads (element i of thread t at [i * S + t]) so a warp's accesses
// to the same field hit 32 consecutive banks.
// ---------------------------------------------------------------------------
// Probability arithmetic of the founder-allele graph.  ProbExact is the
// reference's FP64 (bit-exact); ProbLog2 works on log2 values in FP32 for the
// fast sampler mode, where only the normalised pair of likelihoods is used:
// products become sums and a zero likelihood is -inf.
struct ProbExact {
    using T = double;
    static __device__ __forceinline__ T zero() { return 0.0; }
    static __device__ __forceinline__ T one() { return 1.0; }
    static __device__ __forceinline__ T mul(T a, T b) { return DMUL(a, b); }
    static __device__ __forceinline__ T add(T a, T b) { return DADD(a, b); }
    static __device__ __forceinline__ T from(double x) { return x; }
    static __device__ __forceinline__ bool is_zero(T a) { return a == 0.0; }
};
struct ProbLog2 {
    using T = float;
    static __device__ __forceinline__ T zero() { return -INFINITY; }
    static __device__ __forceinline__ T one() { return 0.f; }
    static __device__ __forceinline__ T mul(T a, T b) { return a + b; }
    static __device__ __forceinline__ T add(T a, T b) {
        if (a == -INFINITY) return b;
        if (b == -INFINITY) return a;
        const T m = fmaxf(a, b), d = fminf(a, b) - m;
        return m + log2f(1.f + exp2f(d));
    }
    static __device__ __forceinline__ T from(double x) { return x > 0.0 ? log2f((float)x) : -INFINITY; }
    static __device__ __forceinline__ bool is_zero(T a) { return a == -INFINITY; }
};

// Founder-allele groups are kept in a union-find whose links carry a swap
// parity: the reference relabels every member of the absorbed component and
// swaps its two allele assignments when merging (combine_components,
// founder_allele_graph4.cc:491-541); here the absorbed component's root is
// linked under the survivor's root with parity = swap, and a member's
// assignment in its group's frame is its stored pair read through the
// accumulated parity.  Group ids, the fixed/active flags and every FP64
// product follow the reference's order exactly, so the likelihood is the
// same double.  IX is uint8_t when 2F <= 255 (founder-allele and group ids
// fit a byte), else uint16_t.
template <typename IX, typename PT>
struct Fag {
    PT* pr0;          // [2F][S] prob[0][group]
    PT* pr1;          // [2F][S]
    IX* edge;         // [2N][S] founder allele of each person's maternal/paternal allele
    IX* up;           // [2F][S] union-find parent of a founder allele
    uint8_t* fl;      // [2F][S] bit0 parity to parent, bit1 in a group, bits 2-3 a0, bits 4-5 a1
    int8_t* fx;       // [2F][S] group fixed: -1 unfixed, 0/1 fixed, 2 inactive
    IX* root;         // [2F][S] root founder allele of a group id
    IX* gid;          // [2F][S] group id of a root founder allele
    int S, t;
    __device__ __forceinline__ PT& p0(int g) { return pr0[g * S + t]; }
    __device__ __forceinline__ PT& p1(int g) { return pr1[g * S + t]; }
    __device__ __forceinline__ PT& pw(int w, int g) { return w == 0 ? p0(g) : p1(g); }
    __device__ __forceinline__ IX& e(int i) { return edge[i * S + t]; }
};

__host__ __device__ inline size_t fag_per_thread(int N, int F, int fast) {
    const size_t ix = (2 * F <= 255) ? 1 : 2;
    const size_t pb = fast ? 4 : 8;
    return (size_t)2 * F * 2 * pb + (size_t)2 * N * ix + (size_t)2 * F * (3 * ix + 2);
}

// Shared bytes of a block of S threads: the FAG arrays plus the staged
// person tables (order, mother, father as int16 and typed as uint8).
__host__ __device__ inline size_t fag_block_bytes(int N, int F, int S, int fast) {
    size_t tables = ((size_t)N * 7 + 15) & ~(size_t)15;
    return ((fag_per_thread(N, F, fast) * S + 15) & ~(size_t)15) + tables;
}

template <typename IX, typename PT>
__device__ __forceinline__ Fag<IX, PT> fag_bind(unsigned char* p, int N, int F, int S, int t) {
    Fag<IX, PT> s;
    s.S = S;
    s.t = t;
    s.pr0 = (PT*)p;
    s.pr1 = s.pr0 + (size_t)2 * F * S;
    s.edge = (IX*)(s.pr1 + (size_t)2 * F * S);
    s.up = s.edge + (size_t)2 * N * S;
    s.root = s.up + (size_t)2 * F * S;
    s.gid = s.root + (size_t)2 * F * S;
    s.fl = (uint8_t*)(s.gid + (size_t)2 * F * S);
    s.fx = (int8_t*)(s.fl + (size_t)2 * F * S);
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

// Root of a founder allele's component and the parity from the allele to it,
// compressing the path.
template <typename FS>
__device__ __forceinline__ int fag_find(FS& s, int fa, int& parity) {
    int r = fa, p = 0;
    while (true) {
        const int u = s.up[r * s.S + s.t];
        if (u == r) break;
        p ^= s.fl[r * s.S + s.t] & 1;
        r = u;
    }
    int x = fa, px = p;
    while (x != r) {
        const int u = s.up[x * s.S + s.t];
        const uint8_t f = s.fl[x * s.S + s.t];
        s.up[x * s.S + s.t] = r;
        s.fl[x * s.S + s.t] = (uint8_t)((f & ~1) | px);
        px ^= f & 1;
        x = u;
    }
    parity = p;
    return r;
}

// A founder allele as the reference sees it: its group id (-1 = none) and its
// two allele assignments in its group's frame.
struct FaView {
    int group, a0, a1;
    __device__ __forceinline__ int a(int w) const { return w ? a1 : a0; }
};

template <typename FS>
__device__ __forceinline__ FaView fag_view(FS& s, int fa) {
    FaView v;
    const uint8_t f = s.fl[fa * s.S + s.t];
    if (!(f & 2)) { v.group = -1; v.a0 = v.a1 = 0; return v; }
    int par;
    const int r = fag_find(s, fa, par);
    const uint8_t g = s.fl[fa * s.S + s.t];
    const int s0 = (g >> 2) & 3, s1 = (g >> 4) & 3;
    v.group = s.gid[r * s.S + s.t];
    v.a0 = par ? s1 : s0;
    v.a1 = par ? s0 : s1;
    return v;
}

// Put founder allele fa in group g with assignment value `val` in slot w (the
// other slot unset, as in the reference), linked straight to the group's root.
template <typename FS>
__device__ __forceinline__ void fag_join(FS& s, int fa, int g, int w, int val) {
    const int r = s.root[g * s.S + s.t];
    s.up[fa * s.S + s.t] = r;
    s.fl[fa * s.S + s.t] = (uint8_t)(2 | (val << (w == 0 ? 2 : 4)));
}

template <typename FS>
__device__ __forceinline__ void fag_join2(FS& s, int fa, int g, int v0, int v1) {
    const int r = s.root[g * s.S + s.t];
    s.up[fa * s.S + s.t] = r;
    s.fl[fa * s.S + s.t] = (uint8_t)(2 | (v0 << 2) | (v1 << 4));
}

template <typename FS>
__device__ __forceinline__ void fag_new_root(FS& s, int fa, int g, int v0, int v1) {
    s.up[fa * s.S + s.t] = fa;
    s.fl[fa * s.S + s.t] = (uint8_t)(2 | (v0 << 2) | (v1 << 4));
    s.root[g * s.S + s.t] = fa;
    s.gid[fa * s.S + s.t] = g;
}

// combine_components(c1, c2, flip) (founder_allele_graph4.cc:491-541)
template <typename PP, typename FS>
__device__ __forceinline__ void fag_combine(FS& s, int c1, int c2, bool flip) {
    const int r1 = s.root[c1 * s.S + s.t], r2 = s.root[c2 * s.S + s.t];
    s.up[r2 * s.S + s.t] = r1;
    s.fl[r2 * s.S + s.t] = (uint8_t)((s.fl[r2 * s.S + s.t] & ~1) | (flip ? 1 : 0));
    if (flip) {
        s.p0(c1) = PP::mul(s.p0(c1), s.p1(c2));
        s.p1(c1) = PP::mul(s.p1(c1), s.p0(c2));
    } else {
        s.p0(c1) = PP::mul(s.p0(c1), s.p0(c2));
        s.p1(c1) = PP::mul(s.p1(c1), s.p1(c2));
    }
    s.fx[c2 * s.S + s.t] = 2;
}

// Edges of the column (FounderAlleleGraph4::reset, founder_allele_graph4.cc:
// 543-569) with one meiosis optionally toggled, which equals flip() and its
// propagation (founder_allele_graph4.cc:571-597).
template <typename FS>
__device__ void fag_edges(int N, int F, const int16_t* order, const int16_t* mo, const int16_t* fa,
                          const uint32_t* col, FS& s, int flip_b) {
    for (int n = 0; n < N; ++n) {
        const int pid = order[n];
        if (pid < F) {
            s.e(2 * pid) = 2 * pid;
            s.e(2 * pid + 1) = 2 * pid + 1;
        } else {
            const int b = 2 * (pid - F);
            const int vm = dgbit(col, b) ^ (flip_b == b);
            const int vp = dgbit(col, b + 1) ^ (flip_b == b + 1);
            s.e(2 * pid) = s.e(2 * mo[pid] + vm);
            s.e(2 * pid + 1) = s.e(2 * fa[pid] + vp);
        }
    }
}

template <typename PP, typename FS>
__device__ typename PP::T fag_like(int N, int F, const uint8_t* typed, const uint8_t* gcol, double minor_d, FS& s) {
    using T = typename PP::T;
    const int nfa = 2 * F;
    const T major = PP::from(DSUB(1.0, minor_d)), minor = PP::from(minor_d);
    for (int i = 0; i < nfa; ++i) s.fl[i * s.S + s.t] = 0;
    int gi = 0;
#define FREQ(g) ((g) == G_HOMOZ_A ? major : minor)
#define FX(g) s.fx[(g) * s.S + s.t]
#define ZERO PP::zero()
    for (int i = 0; i < N; ++i) {
        if (!typed[i]) continue;
        const int g = gcol[i] & 3;
        if (g == G_UNTYPED) continue;
        const int mfa = s.e(2 * i), pfa = s.e(2 * i + 1);
        if (mfa == pfa) {
            if (g == G_HETERO) return ZERO;
            const FaView m = fag_view(s, mfa);
            if (m.group != -1) {
                const int g1 = m.group;
                const int f1 = FX(g1);
                if (f1 != -1) {
                    if (g != m.a(f1)) return ZERO;
                } else {
                    if (m.a(0) == g) { FX(g1) = 0; s.p1(g1) = ZERO; }
                    else if (m.a(1) == g) { FX(g1) = 1; s.p0(g1) = ZERO; }
                    else return ZERO;
                }
            } else {
                fag_new_root(s, mfa, gi, g, 0);
                FX(gi) = 0;
                s.p0(gi) = FREQ(g);
                s.p1(gi) = ZERO;
                ++gi;
            }
            continue;
        }
        const FaView m = fag_view(s, mfa);
        const FaView p = fag_view(s, pfa);
        const int g1 = m.group, g2 = p.group;
        if (g1 != -1) {
            int f1 = FX(g1);
            if (g2 != -1) {
                if (g1 == g2) {
                    if (f1 != -1) {
                        if (!fag_legal(g, m.a(f1), p.a(f1))) return ZERO;
                    } else {
                        const int l0 = fag_legal(g, m.a(0), p.a(0));
                        const int l1 = fag_legal(g, m.a(1), p.a(1));
                        if (l0) {
                            if (!l1) { FX(g1) = 0; s.p1(g1) = ZERO; }
                        } else {
                            if (l1) { FX(g1) = 1; s.p0(g1) = ZERO; }
                            else return ZERO;
                        }
                    }
                } else {
                    int f2 = FX(g2);
                    if (f1 != -1) {
                        if (f2 != -1) {
                            if (!fag_legal(g, m.a(f1), p.a(f2))) return ZERO;
                        } else {
                            const int l0 = fag_legal(g, m.a(f1), p.a(0));
                            const int l1 = fag_legal(g, m.a(f1), p.a(1));
                            if (l0) f2 = 0; else if (l1) f2 = 1; else return ZERO;
                        }
                    } else if (f2 != -1) {
                        const int l0 = fag_legal(g, m.a(0), p.a(f2));
                        const int l1 = fag_legal(g, m.a(1), p.a(f2));
                        if (l0) f1 = 0; else if (l1) f1 = 1; else return ZERO;
                    } else {
                        const int l0 = fag_legal(g, m.a(0), p.a(0));
                        const int l1 = fag_legal(g, m.a(1), p.a(0));
                        const int l2 = fag_legal(g, m.a(0), p.a(1));
                        const int l3 = fag_legal(g, m.a(1), p.a(1));
                        if (!(l0 || l1 || l2 || l3)) return ZERO;
                        if (l0 && !(l1 || l2 || l3)) { f1 = 0; f2 = 0; }
                        else if (l1 && !(l0 || l2 || l3)) { f1 = 1; f2 = 0; }
                        else if (l2 && !(l0 || l1 || l3)) { f1 = 0; f2 = 1; }
                        else if (l3 && !(l0 || l1 || l2)) { f1 = 1; f2 = 1; }
                        else if (l0 && l3 && !(l1 || l2)) { f1 = -1; f2 = -1; }
                        else if (l1 && l2 && !(l0 || l3)) { f1 = -2; f2 = -2; }
                        else { f1 = -1; f2 = -1; }
                    }
                    if (f1 != f2) {
                        FX(g1) = (int8_t)f1;
                        s.pw(1 - f1, g1) = ZERO;
                        s.pw(1 - f2, g2) = ZERO;
                        fag_combine<PP>(s, g1, g2, true);
                    } else if (f1 == -2) {
                        FX(g1) = -1;
                        fag_combine<PP>(s, g1, g2, true);
                    } else {
                        FX(g1) = (int8_t)f1;
                        if (f1 != -1) {
                            s.pw(1 - f1, g1) = ZERO;
                            s.pw(1 - f2, g2) = ZERO;
                        }
                        fag_combine<PP>(s, g1, g2, false);
                    }
                }
            } else {
                if (f1 != -1) {
                    const int t0 = fag_other(g, m.a(f1));
                    if (t0 == G_UNTYPED) return ZERO;
                    fag_join(s, pfa, g1, f1, t0);
                    s.pw(f1, g1) = PP::mul(s.pw(f1, g1), FREQ(t0));
                } else {
                    const int t0 = fag_other(g, m.a(0));
                    const int t1 = fag_other(g, m.a(1));
                    if (t0 != G_UNTYPED) {
                        if (t1 != G_UNTYPED) {
                            fag_join2(s, pfa, g1, t0, t1);
                            s.p0(g1) = PP::mul(s.p0(g1), FREQ(t0));
                            s.p1(g1) = PP::mul(s.p1(g1), FREQ(t1));
                        } else {
                            fag_join(s, pfa, g1, 0, t0);
                            s.p0(g1) = PP::mul(s.p0(g1), FREQ(t0));
                            s.p1(g1) = ZERO;
                            FX(g1) = 0;
                        }
                    } else {
                        if (t1 != G_UNTYPED) {
                            fag_join(s, pfa, g1, 1, t1);
                            s.p1(g1) = PP::mul(s.p1(g1), FREQ(t1));
                            s.p0(g1) = ZERO;
                            FX(g1) = 1;
                        } else return ZERO;
                    }
                }
            }
        } else if (g2 != -1) {
            const int f2 = FX(g2);
            if (f2 != -1) {
                const int t0 = fag_other(g, p.a(f2));
                if (t0 == G_UNTYPED) return ZERO;
                fag_join(s, mfa, g2, f2, t0);
                s.pw(f2, g2) = PP::mul(s.pw(f2, g2), FREQ(t0));
            } else {
                const int t0 = fag_other(g, p.a(0));
                const int t1 = fag_other(g, p.a(1));
                if (t0 != G_UNTYPED) {
                    if (t1 != G_UNTYPED) {
                        fag_join2(s, mfa, g2, t0, t1);
                        s.p0(g2) = PP::mul(s.p0(g2), FREQ(t0));
                        s.p1(g2) = PP::mul(s.p1(g2), FREQ(t1));
                    } else {
                        fag_join(s, mfa, g2, 0, t0);
                        s.p0(g2) = PP::mul(s.p0(g2), FREQ(t0));
                        s.p1(g2) = ZERO;
                        FX(g2) = 0;
                    }
                } else {
                    if (t1 != G_UNTYPED) {
                        fag_join(s, mfa, g2, 1, t1);
                        s.p1(g2) = PP::mul(s.p1(g2), FREQ(t1));
                        s.p0(g2) = ZERO;
                        FX(g2) = 1;
                    } else return ZERO;
                }
            }
        } else {
            if (g == G_HETERO) {
                fag_new_root(s, mfa, gi, G_HOMOZ_A, G_HOMOZ_B);
                fag_join2(s, pfa, gi, G_HOMOZ_B, G_HOMOZ_A);
                s.p0(gi) = PP::mul(major, minor);
                s.p1(gi) = PP::mul(major, minor);
                FX(gi) = -1;
            } else {
                fag_new_root(s, mfa, gi, g, 0);
                fag_join(s, pfa, gi, 0, g);
                s.p0(gi) = PP::mul(FREQ(g), FREQ(g));
                s.p1(gi) = ZERO;
                FX(gi) = 0;
            }
            ++gi;
        }
    }
#undef FREQ
    T ret = PP::one();
    for (int i = 0; i < gi; ++i) {
        const int f = FX(i);
        if (f == 2) continue;
        if (f != -1) ret = PP::mul(ret, s.pw(f, i));
        else ret = PP::mul(ret, PP::add(s.p0(i), s.p1(i)));
    }
#undef FX
#undef ZERO
    return ret;
}

// ---------------------------------------------------------------------------
// M-sampler, split per meiosis step into a grid-wide likelihood kernel and a
// per-chain forward-filter / backward-sample kernel (meiosis_sampler.cc:
// 17-203).  raw64[cr][locus][2] holds the exact likelihoods; raw32 holds the
// same pair divided by its larger member, for the FP32 filter.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void put_raw32(float* r32, int l, double v0, double v1) {
    const double mx = v0 > v1 ? v0 : v1;
    float a = 0.f, b = 0.f;
    if (mx > 0.0) {
        a = (float)(v0 / mx);
        b = (float)(v1 / mx);
    }
    r32[2 * l] = a;
    r32[2 * l + 1] = b;
}

__device__ __forceinline__ void put_raw32_log2(float* r32, int l, float l0, float l1) {
    const float mx = fmaxf(l0, l1);
    float a = 0.f, b = 0.f;
    if (mx != -INFINITY) {
        a = l0 == -INFINITY ? 0.f : exp2f(l0 - mx);
        b = l1 == -INFINITY ? 0.f : exp2f(l1 - mx);
    }
    r32[2 * l] = a;
    r32[2 * l + 1] = b;
}

// step < 0: reset at order[0] (raw[l][cur] = likelihood of the column);
// step >= 0: likelihoods of meiosis order[step] at both values.  With
// ProbExact, raw holds the reference's doubles; with ProbLog2 it holds log2
// likelihoods and raw32 receives each pair divided by its larger member.
template <typename IX, typename PP>
__global__ void __launch_bounds__(128) fag_kernel(ProblemDev P, uint32_t* dg, int first, int nchain,
                                                  const int32_t* order, int64_t ostride, int step,
                                                  const uint8_t* sel, int want, typename PP::T* rawbuf,
                                                  float* raw32, uint8_t* badc, int* status, int fast) {
    using T = typename PP::T;
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = blockDim.x;
    const size_t per = fag_block_bytes(P.N, P.F, S, fast) - (((size_t)P.N * 7 + 15) & ~(size_t)15);
    int16_t* s_order = (int16_t*)(smem + per);
    int16_t* s_mo = s_order + P.N;
    int16_t* s_fa = s_mo + P.N;
    uint8_t* s_typed = (uint8_t*)(s_fa + P.N);
    for (int i = threadIdx.x; i < P.N; i += S) {
        s_order[i] = P.fag_order[i];
        s_mo[i] = P.mother[i];
        s_fa[i] = P.father[i];
        s_typed[i] = P.typed[i];
    }
    __syncthreads();
    Fag<IX, T> fs = fag_bind<IX, T>(smem, P.N, P.F, S, threadIdx.x);
    const int64_t ntask = (int64_t)nchain * P.M;
    const int64_t t = (int64_t)blockIdx.x * S + threadIdx.x;
    if (t >= ntask) return;
    const int cr = (int)(t / P.M);
    const int l = (int)(t % P.M);
    if (sel && sel[cr] != want) return;
    const int chain = first + cr;
    const uint32_t* col = dg + ((size_t)chain * P.M + l) * P.W;
    const int32_t* ord = order + cr * ostride;
    T* raw = rawbuf + (size_t)cr * 2 * P.M;
    const uint8_t* gcol = P.geno + (size_t)l * P.N;
    if (step < 0) {
        fag_edges(P.N, P.F, s_order, s_mo, s_fa, col, fs, -1);
        const T lk = fag_like<PP>(P.N, P.F, s_typed, gcol, P.c_minor[(size_t)chain * P.M + l], fs);
        raw[2 * l + dgbit(col, ord[0])] = lk;
        if (PP::is_zero(lk)) {
            badc[cr] = 1;
            set_status(status, ST_ILLEGAL_DG);
        }
        return;
    }
    const int m = ord[step];
    const int last = ord[step > 0 ? step - 1 : 0];
    const int tb = dgbit(col, m), t2 = dgbit(col, last);
    const T keep = raw[2 * l + t2];
    fag_edges(P.N, P.F, s_order, s_mo, s_fa, col, fs, m);
    const T lk = fag_like<PP>(P.N, P.F, s_typed, gcol, P.c_minor[(size_t)chain * P.M + l], fs);
    raw[2 * l + tb] = keep;
    raw[2 * l + 1 - tb] = lk;
    if (raw32) {
        float* r32 = raw32 + (size_t)cr * 2 * P.M;
        if (sizeof(T) == 8) {
            if (tb == 0) put_raw32(r32, l, (double)keep, (double)lk); else put_raw32(r32, l, (double)lk, (double)keep);
        } else {
            if (tb == 0) put_raw32_log2(r32, l, (float)keep, (float)lk);
            else put_raw32_log2(r32, l, (float)lk, (float)keep);
        }
    }
    if (PP::is_zero(keep) && PP::is_zero(lk)) {
        badc[cr] = 1;
        set_status(status, ST_ILLEGAL_DG);
    }
}

// ---------------------------------------------------------------------------
// Fast-mode founder-allele-graph likelihood, one group of G lanes (a warp, or
// half a warp) per (chain, locus).  The likelihood of the genotypes given the
// column's founder-allele graph (FounderAlleleGraph4::likelihood,
// founder_allele_graph4.cc:34-442) is the product over the connected
// components of the heterozygote edges of the sum, over the component's two
// colourings (allele A = major, B = minor) that satisfy every homozygote's
// fixed alleles, of the product of the founder alleles' frequencies.  Here:
//   1. the founder allele of every person's two alleles is propagated one
//      generation level at a time, the lanes splitting a level's persons;
//   2. the locus's typed persons (a list built at context creation,
//      heterozygotes first) mark their founder alleles used / fixed A /
//      fixed B (shared-memory atomicOr); a heterozygote on one founder allele
//      is a zero likelihood;
//   3. the heterozygote edges join components in a lock-free union-find with
//      parities (pf_find; a compare-and-swap hooks the larger root under the
//      smaller, so every root is its component's smallest allele whatever the
//      interleaving); an edge whose ends already share a root with equal
//      parity closes an odd cycle: zero;
//   4. a component's two colourings weigh (even members) x log2 f(A) + (odd
//      members) x log2 f(B) and the reverse, so each component needs only
//      integer counts, taken at its root; a butterfly sum over the group
//      gives log2 of the likelihood.
// ---------------------------------------------------------------------------
constexpr int kFagWarpsPerBlock = 8;
constexpr int kFagRounds = 4;   // rounds of colour propagation along heterozygote edges

__host__ __device__ inline size_t fagw_tables(int N) {
    return (((size_t)N * 8 + 15) & ~(size_t)15) + (((size_t)4 * (N + 1) + 15) & ~(size_t)15);
}
// per lane group: e [2N] founder-allele labels of eb bytes each (1 when the
// 2F labels fit a byte: less shared memory per block, more blocks per SM),
// then Lb / fl / cnt [2F] int each, then the typed-member list [N] u16 on a
// 16-byte boundary in whole 16-byte chunks
__host__ __device__ inline size_t fagw_typ_offset(int N, int F, int eb) {
    return (((((size_t)2 * eb * N + 15) & ~(size_t)15) + (size_t)2 * F * 12) + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t fagw_warp_bytes(int N, int F, int eb) {
    return fagw_typ_offset(N, F, eb) + (size_t)16 * ((N + 7) / 8);
}
// per block: the shared tables and one locus's arrays per lane group (G lanes)
size_t fagw_block_bytes(int N, int F, int G, int eb) {
    return fagw_tables(N) + (size_t)kFagWarpsPerBlock * (32 / G) * fagw_warp_bytes(N, F, eb);
}
// bytes of a founder-allele label: one while the 2F labels fit
__host__ __device__ inline int fagw_label_bytes(int F) { return 2 * F <= 256 ? 1 : 2; }

// 16-byte global -> shared copies that complete asynchronously (cp.async,
// sm_80 and later): both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Root of founder allele x in a forest of 2 * parent + parity entries, and
// x's parity to it.  Parents have smaller indices than their children, so the
// walk ends within x steps.  On the way every other entry is pointed at its
// grandparent with the composed parity (path halving): only entries that are
// not roots are rewritten, always to an ancestor, so the forest stays valid
// whatever other lanes do meanwhile.
__device__ __forceinline__ int pf_find(volatile int* L, int x, int& parity) {
    int p = 0, y = x;
    for (int it = 0; it < 8192; ++it) {
        const int v = L[y];
        const int up = v >> 1;
        if (up == y) break;
        const int w = L[up];
        const int gp = w >> 1;
        if (gp == up) {   // up is the root
            p ^= v & 1;
            y = up;
            break;
        }
        const int pg = (v ^ w) & 1;   // parity of y to its grandparent
        L[y] = (gp << 1) | pg;
        p ^= pg;
        y = gp;
    }
    parity = p;
    return y;
}

// The tables every warp of a block shares, loaded into the block's shared memory.
struct FagwTables {
    uint2* lvl;         // [N] members by generation level: x = member, y = 2 mother | 2 father << 16
    int32_t* lvl_off;   // [n_lvl + 1]
};

__device__ FagwTables fagw_load_tables(const ProblemDev& P, unsigned char* smem) {
    const int N = P.N;
    FagwTables t;
    t.lvl = (uint2*)smem;
    t.lvl_off = (int32_t*)(smem + (((size_t)N * 8 + 15) & ~(size_t)15));
    for (int q = threadIdx.x; q < N; q += blockDim.x) {
        const int pid = P.lvl_order[q];
        const int mo = P.mother[pid], fa = P.father[pid];
        t.lvl[q] = make_uint2((unsigned)pid, mo < 0 ? 0u : (unsigned)(2 * mo) | ((unsigned)(2 * fa) << 16));
    }
    for (int i = threadIdx.x; i <= P.n_lvl; i += blockDim.x) t.lvl_off[i] = P.lvl_off[i];
    return t;
}

// A group of G lanes (32 or 16) of a warp, aligned, working on one locus;
// every primitive runs on the full warp and is read per group.
template <int G>
struct LaneGroup {
    int gl, base;
    __device__ LaneGroup() {
        const int lane = threadIdx.x & 31;
        gl = lane & (G - 1);
        base = lane & ~(G - 1);
    }
    __device__ __forceinline__ unsigned ballot(bool p) const {
        const unsigned b = __ballot_sync(FULLMASK, p);
        return G == 32 ? b : (b >> base) & ((1u << G) - 1u);
    }
    __device__ __forceinline__ bool any(bool p) const { return ballot(p) != 0u; }
    __device__ __forceinline__ uint32_t shfl(uint32_t v, int src) const { return __shfl_sync(FULLMASK, v, src, G); }
};

// One (chain, locus) task by one group of G lanes (32 / G loci per warp, in
// lockstep: every loop below has the same trip count in all groups except the
// union loop, which holds no warp primitive).  step < 0 stores the likelihood
// of the column at meiosis order[0]; step >= 0 the likelihoods at both values
// of meiosis order[step] (the kept one from the previous step).  A group past
// the last locus (valid false) works on locus 0 and stores nothing.
template <int G, typename E>
__device__ __forceinline__ void fagw_task(const ProblemDev& P, const FagwTables& tab, unsigned char* wbase,
                                          const uint32_t* dg, int chain, int cr, int l, bool valid,
                                          const int32_t* ord, int step, float* rawbuf, float* raw32, uint8_t* badc,
                                          int* status) {
    const LaneGroup<G> grp;
    const int N = P.N, F = P.F, nfa = 2 * F, M = P.M, gl = grp.gl;
    const uint2* s_lvl = tab.lvl;
    const int32_t* s_off = tab.lvl_off;
    E* e = (E*)wbase;                                                 // [2N] founder allele of each allele
    volatile int* Lb = (volatile int*)(wbase + (((size_t)2 * sizeof(E) * N + 15) & ~(size_t)15));   // [2F] 2 * parent + parity
    int* fl = (int*)(Lb + nfa);                                       // [2F] bit0 used, bit1 fixed A, bit2 fixed B
    int* cnt = fl + nfa;                                              // [2F] per component: counts, forbidden colourings
    uint16_t* typ = (uint16_t*)(wbase + fagw_typ_offset(N, F, (int)sizeof(E)));   // [N] the locus's typed members
    const int lc = valid ? l : 0;
    const uint32_t* col = dg + ((size_t)chain * M + lc) * P.W;
    float* raw = rawbuf + (size_t)cr * 2 * M;
    // the task's global reads issued together: the column's words (lane w of
    // the group holds word w, read by shuffles), the allele frequencies'
    // log2, and the locus's typed members (member << 2 | genotype code,
    // heterozygotes first: fixed by the genotypes, listed once at context
    // creation), copied to shared memory in 16-byte asynchronous copies that
    // complete while the founder alleles are propagated
    const bool wreg = P.W <= G;
    const uint32_t cw = wreg && gl < P.W ? col[gl] : 0u;
    const int t0 = P.typ_off[lc], ntyp = P.typ_cnt[lc], nhet = P.typ_nhet[lc];
    const float2 lfreq = P.c_lfreq[(size_t)chain * M + lc];
    for (int q = gl; q < (ntyp + 7) >> 3; q += G) cp_async16(typ + 8 * q, P.typ_ent + t0 + 8 * q);
    cp_async_commit();
    auto cbit = [&](int b) -> int {
        const uint32_t w = wreg ? grp.shfl(cw, b >> 5) : col[b >> 5];
        return (int)((w >> (b & 31)) & 1u);
    };
    int flip = -1, tb = 0;
    float keep = 0.f;
    if (step >= 0) {
        const int m = ord[step];
        const int last = ord[step > 0 ? step - 1 : 0];
        tb = cbit(m);
        keep = raw[2 * lc + cbit(last)];
        flip = m;
    }
    // 1. founder alleles, one generation level at a time
    for (int q = gl; q < s_off[1]; q += G) {
        const int pid = (int)s_lvl[q].x;
        e[2 * pid] = (E)(2 * pid);
        e[2 * pid + 1] = (E)(2 * pid + 1);
    }
    __syncwarp();
    for (int k = 1; k < P.n_lvl; ++k) {
        // every lane takes part in the shuffles, members or not
        for (int q0 = s_off[k]; q0 < s_off[k + 1]; q0 += G) {
            const int q = q0 + gl;
            const bool act = q < s_off[k + 1];
            const uint2 ent = act ? s_lvl[q] : make_uint2((unsigned)F, 0u);
            const int pid = (int)ent.x;
            const int b = 2 * (pid - F);
            const uint32_t w = wreg ? grp.shfl(cw, b >> 5) : col[b >> 5];
            if (!act) continue;
            const int vm = (int)((w >> (b & 31)) & 1u) ^ (flip == b);
            const int vp = (int)((w >> ((b + 1) & 31)) & 1u) ^ (flip == b + 1);
            e[2 * pid] = e[(ent.y & 0xffffu) + vm];
            e[2 * pid + 1] = e[(ent.y >> 16) + vp];
        }
        __syncwarp();
    }
    // 2. fixed founder alleles: the homozygous typed members (after the
    // heterozygotes in the list) mark theirs with the colour their genotype
    // forces (no warp primitive inside: the groups' loci have lists of their
    // own lengths)
    for (int x = gl; x < nfa; x += G) {
        Lb[x] = x << 1;
        fl[x] = 0;
        cnt[x] = 0;
    }
    cp_async_wait_all();   // this lane's copies of the list; the barrier makes the group's visible
    __syncwarp();
    for (int x = nhet + gl; x < ntyp; x += G) {
        const int ent = typ[x], i = ent >> 2, g = ent & 3;
        const int bits = g == G_HOMOZ_A ? 3 : 5;   // used, fixed A / fixed B
        atomicOr(&fl[e[2 * i]], bits);
        atomicOr(&fl[e[2 * i + 1]], bits);
    }
    __syncwarp();
    // 3. components of the heterozygote edges with parities: a lock-free
    // union-find forest in Lb (2 * parent + parity to the parent), each lane
    // joining its edges by hooking the larger root under the smaller with a
    // compare-and-swap (so a root is its component's smallest allele); an edge
    // whose ends already share a root must have ends of opposite parity.  A
    // failed hook means another lane's hook succeeded, so a lane retries fewer
    // than 2F times.  An edge whose two ends are both fixed only needs their
    // colours to differ: the two sides' colourings are then determined apart,
    // and the likelihood is the product of the two sides' terms, so the edge
    // joins nothing.  The ends of the other edges are marked used and joined
    // (bit 3: in the forest).  First, a heterozygote with exactly one fixed
    // end fixes the other to the opposite colour, in rounds until nothing
    // changes (at most kFagRounds): most edges then have both ends fixed, and
    // a fixed allele's colour is its component's, so its term is the same.
    for (int round = 0; round < kFagRounds; ++round) {
        int changed = 0;
        for (int q = gl; q < nhet; q += G) {
            const int i = typ[q] >> 2;
            const int u = e[2 * i], v = e[2 * i + 1];
            const int fu = fl[u] & 6, fv = fl[v] & 6;
            if ((fu != 0) == (fv != 0)) continue;   // both ends fixed, or neither
            const int cf = fu ? fu : fv;
            const int opp = cf == 2 ? 4 : (cf == 4 ? 2 : 6);
            atomicOr(&fl[fu ? v : u], opp | 1);
            changed = 1;
        }
        __syncwarp();
        if (!__any_sync(FULLMASK, changed)) break;   // the whole warp, as its groups share the loop
    }
    int bad = 0;
    for (int q = gl; q < nhet; q += G) {
        const int i = typ[q] >> 2;   // the heterozygotes lead the list
        const int u = e[2 * i], v = e[2 * i + 1];
        if (u == v) {   // one founder allele cannot give both alleles of a heterozygote
            bad = 1;
            continue;
        }
        const int fu = fl[u], fv = fl[v];
        if ((fu & 6) && (fv & 6)) {
            if (fu & fv & 6) bad = 1;   // both ends forced to the same colour
            continue;
        }
        atomicOr(&fl[u], 9);
        atomicOr(&fl[v], 9);
        for (int tries = 0;; ++tries) {
            if (tries > nfa) {
                bad = 1;
                set_status(status, ST_ILLEGAL_DG);
                break;
            }
            int pu, pv;
            const int ru = pf_find(Lb, u, pu), rv = pf_find(Lb, v, pv);
            if (ru == rv) {
                if ((pu ^ pv) != 1) bad = 1;   // an odd cycle of heterozygote edges
                break;
            }
            const int lo = min(ru, rv), hi = max(ru, rv);
            if (atomicCAS((int*)&Lb[hi], hi << 1, (lo << 1) | (pu ^ pv ^ 1)) == (hi << 1)) break;
        }
    }
    bad = grp.any(bad);
    __syncwarp();
    // 4. sum over each component's colourings, log2: every member allele
    // contributes log2 of the major or the minor frequency, so a component
    // needs only its member count, how many members have even parity and
    // which colourings its fixed members forbid (integer shared-memory
    // atomics, the same result in any order).  A fixed allele outside the
    // forest is a component of its own: its term is added directly.
    float sum = 0.f;
    int zero = 0, forest = 0;
    const float lmaj = lfreq.x, lmin = lfreq.y;
    if (!bad)
        for (int x = gl; x < nfa; x += G) {
            const int f = fl[x];
            if (!(f & 1)) continue;
            if (!(f & 8)) {
                if ((f & 6) == 6) zero = 1;
                else sum += (f & 2) ? lmaj : lmin;
                continue;
            }
            forest = 1;
            int p = 0;
            const int r = pf_find(Lb, x, p);   // the forest is final: the unions are done
            // bit 16 + n: member count; bits 0-15: even-parity members; bits 29/30: colouring 0/1 forbidden
            const int add = (1 << 16) + (p ? 0 : 1);
            int forbid = 0;
            if (f & 2) forbid |= p ? (1 << 29) : (1 << 30);   // fixed A
            if (f & 4) forbid |= p ? (1 << 30) : (1 << 29);   // fixed B
            atomicAdd(&cnt[r], add);
            if (forbid) atomicOr(&cnt[r], forbid);
        }
    forest = grp.any(forest);   // no union: every term is in already
    __syncwarp();
    if (!bad && forest) {
        for (int x = gl; x < nfa; x += G) {
            const int c = cnt[x];
            const int n = (c >> 16) & 0x1fff, even = c & 0xffff;
            if (n == 0) continue;
            const float w0 = (float)even * lmaj + (float)(n - even) * lmin;   // root coloured A
            const float w1 = (float)even * lmin + (float)(n - even) * lmaj;   // root coloured B
            const int ok0 = !(c & (1 << 29)), ok1 = !(c & (1 << 30));
            if (ok0 && ok1) {
                const float mx = fmaxf(w0, w1);
                sum += mx + log2f(1.f + exp2f(fminf(w0, w1) - mx));
            } else if (ok0) sum += w0;
            else if (ok1) sum += w1;
            else zero = 1;
        }
    }
    zero = grp.any(zero);
    for (int dd = G / 2; dd >= 1; dd >>= 1) sum += __shfl_xor_sync(FULLMASK, sum, dd);
    const float lk = (bad || zero) ? -INFINITY : sum;
    if (gl == 0 && valid) {
        if (step < 0) {
            raw[2 * l + dgbit(col, ord[0])] = lk;
            if (lk == -INFINITY) {
                badc[cr] = 1;
                set_status(status, ST_ILLEGAL_DG);
            }
        } else {
            raw[2 * l + tb] = keep;
            raw[2 * l + 1 - tb] = lk;
            float* r32 = raw32 + (size_t)cr * 2 * M;
            if (tb == 0) put_raw32_log2(r32, l, keep, lk);
            else put_raw32_log2(r32, l, lk, keep);
            if (keep == -INFINITY && lk == -INFINITY) {
                badc[cr] = 1;
                set_status(status, ST_ILLEGAL_DG);
            }
        }
    }
    __syncwarp();
}

template <typename T>
struct Flt;
template <>
struct Flt<double> {
    static __device__ __forceinline__ double mul(double a, double b) { return DMUL(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return DADD(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return DSUB(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return DDIV(a, b); }
};
template <>
struct Flt<float> {
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
};

// One warp per chain.  All 32 lanes run the same serial recursion on values
// broadcast by shuffles from coalesced 32-locus chunks (the FP64 pipe costs
// the same per warp instruction whatever the active mask).  T=double is the
// reference's arithmetic; T=float is the fast filter on normalised pairs.
template <typename T>
__global__ void __launch_bounds__(32) ffbs_kernel(ProblemDev P, uint32_t* dg, int first, int nchain,
                                                  const int32_t* order, int64_t ostride, int step, Draws draws,
                                                  const uint8_t* sel, int want, const uint8_t* badc,
                                                  const double* raw64, const float* raw32, T* fbbuf) {
    using Fl = Flt<T>;
    const int cr = blockIdx.x;
    if (cr >= nchain) return;
    if (sel && sel[cr] != want) return;
    if (badc[cr]) return;
    const int lane = threadIdx.x;
    const int chain = first + cr;
    const int m = order[cr * ostride + step];
    uint32_t* G = dg + (size_t)chain * P.M * P.W;
    T* fb = fbbuf + (size_t)cr * 2 * P.M;
    const double* r64 = raw64 + (size_t)cr * 2 * P.M;
    const float* r32 = raw32 ? raw32 + (size_t)cr * 2 * P.M : nullptr;
    // forward filter (meiosis_sampler.cc:136-155)
    T prev0 = (T)0, prev1 = (T)0;
    for (int base = 0; base < P.M; base += 32) {
        const int i = base + lane;
        T q0 = (T)0, q1 = (T)0, th = (T)0;
        if (i < P.M) {
            if (sizeof(T) == 8) { q0 = (T)r64[2 * i]; q1 = (T)r64[2 * i + 1]; }
            else { q0 = (T)r32[2 * i]; q1 = (T)r32[2 * i + 1]; }
            if (i >= 1) th = (T)P.c_theta[(size_t)chain * (P.M - 1) + i - 1];
        }
        const int n = min(32, P.M - base);
        T k0 = (T)0, k1 = (T)0;
        for (int x = 0; x < n; ++x) {
            const T a0 = __shfl_sync(FULLMASK, q0, x), a1 = __shfl_sync(FULLMASK, q1, x);
            const T tx = __shfl_sync(FULLMASK, th, x);
            T f0, f1;
            if (base + x == 0) {
                const T tot = Fl::add(a0, a1);
                f0 = Fl::div(a0, tot);
                f1 = Fl::div(a1, tot);
            } else {
                const T ax = Fl::sub((T)1, tx);
                f0 = Fl::mul(a0, Fl::add(Fl::mul(prev1, tx), Fl::mul(prev0, ax)));
                f1 = Fl::mul(a1, Fl::add(Fl::mul(prev0, tx), Fl::mul(prev1, ax)));
                const T tt = Fl::add(f0, f1);
                f0 = Fl::div(f0, tt);
                f1 = Fl::div(f1, tt);
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
        const T f0 = in ? fb[2 * i] : (T)0, f1 = in ? fb[2 * i + 1] : (T)0;
        const T th = (in && i < P.M - 1) ? (T)P.c_theta[(size_t)chain * (P.M - 1) + i] : (T)0;
        uint32_t* wp = in ? (G + (size_t)i * P.W + (m >> 5)) : nullptr;
        const int cur = in ? (int)((*wp >> (m & 31)) & 1u) : 0;
        const int64_t c0 = cursor;
        const double dr = (c0 + lane < P.M) ? draws.get(cr, chain, step, c0 + lane) : 0.0;
        int mine = cur;
        for (int x = 0; x < n; ++x) {
            const int ii = top - x;
            T a0 = __shfl_sync(FULLMASK, f0, x), a1 = __shfl_sync(FULLMASK, f1, x);
            const T tx = __shfl_sync(FULLMASK, th, x);
            if (ii < P.M - 1) {
                const T ax = Fl::sub((T)1, tx);
                a0 = Fl::mul(a0, nxt != 0 ? tx : ax);
                a1 = Fl::mul(a1, nxt != 1 ? tx : ax);
            }
            int samp;
            if (a0 == (T)0) samp = 1;
            else if (a1 == (T)0) samp = 0;
            else {
                const double r = __shfl_sync(FULLMASK, dr, (int)(cursor - c0));
                ++cursor;
                samp = (r < (double)Fl::div(a0, Fl::add(a0, a1))) ? 0 : 1;
            }
            nxt = samp;
            if (lane == x) mine = samp;
        }
        if (in && mine != cur) *wp ^= (1u << (m & 31));
    }
}

// Fast M-sampler filter and sampling in O(M/32 + log 32) depth per chain.
// The forward filter f_i = normalise(diag(r_i) T_i f_{i-1}) is a product of
// 2x2 matrices: each lane multiplies its chunk's matrices, a warp scan
// combines the chunk products, and each lane then replays its chunk from the
// vector entering it.  Backward sampling s_i = d_i(s_{i+1}) is a composition
// of maps {0,1} -> {0,1} (2 bits each: the decision when s_{i+1} = 0 and when
// it is 1), scanned the same way from the top locus down.  A locus consumes a
// draw only when neither filtered probability is zero (meiosis_sampler.cc:
// 193-203), so draw indices come from a suffix count of such loci.
__device__ __forceinline__ void mat_norm(float& a, float& b, float& c, float& d) {
    const float mx = fmaxf(fmaxf(fabsf(a), fabsf(b)), fmaxf(fabsf(c), fabsf(d)));
    if (mx > 0.f) {
        const float inv = 1.f / mx;
        a *= inv; b *= inv; c *= inv; d *= inv;
    }
}

// (x o y)(v) = x(y(v)) for 2-bit maps
__device__ __forceinline__ int map_compose(int x, int y) {
    const int y0 = y & 1, y1 = (y >> 1) & 1;
    return ((x >> y0) & 1) | (((x >> y1) & 1) << 1);
}

// Block-wide scan scratch of ffbs_scan_kernel (blockDim.x = T, a multiple of 32, <= 1024).
struct ScanScratch {
    float4* incl;   // [T] each thread's inclusive filter product
    float4* wmat;   // [32] warp products, then their inclusive scan
    int* wcnt;      // [32] draws per warp
    int* wmap;      // [33] warp decision maps, then their suffix compositions
};

__device__ __forceinline__ void mat_mul_left(float& p00, float& p01, float& p10, float& p11, float o00, float o01,
                                             float o10, float o11) {
    // p <- p * o (o is the earlier product, applied first)
    const float n00 = p00 * o00 + p01 * o10, n01 = p00 * o01 + p01 * o11;
    const float n10 = p10 * o00 + p11 * o10, n11 = p10 * o01 + p11 * o11;
    p00 = n00; p01 = n01; p10 = n10; p11 = n11;
}

// Fast-mode forward filter and backward sampling of one meiosis over all loci,
// one block per chain (meiosis_sampler.cc:123-203 restated as scans): each
// thread owns a run of L = ceil(M / T) loci.
//   forward:  the filter is a product of 2x2 matrices A_i = diag(r_i) R(theta_i);
//             chunk products are scanned across the block (later chunks on the
//             left, normalised to a maximum of 1), and each chunk then filters
//             its loci from the vector entering it;
//   backward: loci draw from M-1 down, a locus drawing when both filtered
//             entries are non-zero; a suffix sum of the chunks' draw counts
//             gives each chunk its first draw, so all draws are generated in
//             parallel; each locus's choice given the locus above is a 2-bit
//             map, and a suffix composition of the chunks' maps gives each
//             chunk the state entering it from above.
// The body for chain `chain` (relative index cr), meiosis m, run by a whole
// block.  upre (may be null) holds the step's draws by index, precomputed;
// with cg, the pairs and draws written by other blocks of the same launch are
// read past L1.
__device__ __forceinline__ void ffbs_scan_chain(const ProblemDev& P, uint32_t* dg, int chain, int cr, int m, int step,
                                const Draws& draws, const double* upre, const float* r, float* fb, uint8_t* maps,
                                int staged, bool cg, unsigned char* fsm) {
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    const int M = P.M;
    uint32_t* G = dg + (size_t)chain * M * P.W;
    float* th = nullptr;        // theta as floats, [M]
    uint32_t* words = nullptr;  // the meiosis's descent-graph word at each locus, [M]
    ScanScratch sc;
    sc.incl = (float4*)fsm;
    sc.wmat = sc.incl + T;
    sc.wcnt = (int*)(sc.wmat + 32);
    sc.wmap = sc.wcnt + 32;
    unsigned char* stage = (unsigned char*)(sc.wmap + 36);
    if (staged) {
        // [r: 2M][fb: 2M][theta: M] floats, [words: M], [maps: M bytes]
        float* sr = (float*)stage;
        float* sfb = sr + 2 * M;
        th = sfb + 2 * M;
        words = (uint32_t*)(th + M);
        uint8_t* smaps = (uint8_t*)(words + M);
        for (int i = tid; i < M; i += T) words[i] = G[(size_t)i * P.W + (m >> 5)];
        for (int i = tid; i < 2 * M; i += T) sr[i] = cg ? __ldcg(r + i) : r[i];
        for (int i = tid; i < M; i += T) th[i] = i > 0 ? P.c_theta_f[(size_t)chain * (M - 1) + i - 1] : 0.f;
        r = sr;
        fb = sfb;
        maps = smaps;
    }
    __syncthreads();
    auto tof = [&](int i) { return th ? th[i] : (i > 0 ? P.c_theta_f[(size_t)chain * (M - 1) + i - 1] : 0.f); };
    const bool rcg = cg && !staged;   // the pairs still in global memory, written by other blocks
    auto rq = [&](int i) { return rcg ? __ldcg(r + i) : r[i]; };
    const int L = (M + T - 1) / T;
    const int s0 = min(M, tid * L), s1 = min(M, s0 + L);
    // chunk product P = A_{s1-1} ... A_{s0} (A_0 = diag(r_0)); an empty chunk is the identity
    float p00 = 1.f, p01 = 0.f, p10 = 0.f, p11 = 1.f;
    for (int i = s0; i < s1; ++i) {
        const float q0 = rq(2 * i), q1 = rq(2 * i + 1);
        const float t = tof(i), a = 1.f - t;
        const float n00 = q0 * (a * p00 + t * p10), n01 = q0 * (a * p01 + t * p11);
        const float n10 = q1 * (t * p00 + a * p10), n11 = q1 * (t * p01 + a * p11);
        p00 = n00; p01 = n01; p10 = n10; p11 = n11;
        // each pair is scaled to a maximum of 1, so 8 steps cannot underflow
        if (((i - s0) & 7) == 7) mat_norm(p00, p01, p10, p11);
    }
    mat_norm(p00, p01, p10, p11);
    // inclusive scan within the warp: S_k = P_k ... P_first
    for (int d = 1; d < 32; d <<= 1) {
        const float o00 = __shfl_up_sync(FULLMASK, p00, d), o01 = __shfl_up_sync(FULLMASK, p01, d);
        const float o10 = __shfl_up_sync(FULLMASK, p10, d), o11 = __shfl_up_sync(FULLMASK, p11, d);
        if (lane >= d) {
            mat_mul_left(p00, p01, p10, p11, o00, o01, o10, o11);
            mat_norm(p00, p01, p10, p11);
        }
    }
    if (lane == 31) sc.wmat[warp] = make_float4(p00, p01, p10, p11);
    __syncthreads();
    if (warp == 0) {
        // inclusive scan of the warp products (nw <= 32)
        float4 w = lane < nw ? sc.wmat[lane] : make_float4(1.f, 0.f, 0.f, 1.f);
        for (int d = 1; d < 32; d <<= 1) {
            const float o00 = __shfl_up_sync(FULLMASK, w.x, d), o01 = __shfl_up_sync(FULLMASK, w.y, d);
            const float o10 = __shfl_up_sync(FULLMASK, w.z, d), o11 = __shfl_up_sync(FULLMASK, w.w, d);
            if (lane >= d) {
                mat_mul_left(w.x, w.y, w.z, w.w, o00, o01, o10, o11);
                mat_norm(w.x, w.y, w.z, w.w);
            }
        }
        __syncwarp();
        if (lane < nw) sc.wmat[lane] = w;
    }
    __syncthreads();
    if (warp > 0) {
        const float4 o = sc.wmat[warp - 1];
        mat_mul_left(p00, p01, p10, p11, o.x, o.y, o.z, o.w);
        mat_norm(p00, p01, p10, p11);
    }
    sc.incl[tid] = make_float4(p00, p01, p10, p11);
    __syncthreads();
    // vector entering the chunk: S_{k-1} (1, 1)
    float v0 = 1.f, v1 = 1.f;
    if (tid > 0) {
        const float4 e = sc.incl[tid - 1];
        v0 = e.x + e.y;
        v1 = e.z + e.w;
    }
    int cnt = 0;
    for (int i = s0; i < s1; ++i) {
        const float q0 = rq(2 * i), q1 = rq(2 * i + 1);
        const float t = tof(i), a = 1.f - t;
        float f0 = q0 * (a * v0 + t * v1), f1 = q1 * (t * v0 + a * v1);
        const float tot = f0 + f1;
        if (tot > 0.f) { const float inv = 1.f / tot; f0 *= inv; f1 *= inv; }
        // keep the reference's exact zeros: a zero likelihood stays zero
        if (q0 == 0.f) f0 = 0.f;
        if (q1 == 0.f) f1 = 0.f;
        fb[2 * i] = f0;
        fb[2 * i + 1] = f1;
        cnt += (f0 != 0.f && f1 != 0.f);
        v0 = f0;
        v1 = f1;
    }
    // draws consumed by loci in higher chunks: a suffix sum over the block
    int x = cnt;
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_down_sync(FULLMASK, x, d);
        if (lane + d < 32) x += y;
    }
    if (lane == 0) sc.wcnt[warp] = x;
    __syncthreads();
    int above = x - cnt;
    for (int w = warp + 1; w < nw; ++w) above += sc.wcnt[w];
    // per-locus decision maps and the chunk's composed map; the chunk's draws are
    // independent of one another, so they are generated four at a time
    int gmap = 2;  // identity: bit0 = 0, bit1 = 1
    int idx = above;
    double ubuf[4];
    int ub = 4;
    for (int i = s1 - 1; i >= s0; --i) {
        const float f0 = fb[2 * i], f1 = fb[2 * i + 1];
        int dmap;
        if (f0 == 0.f) dmap = 3;
        else if (f1 == 0.f) dmap = 0;
        else {
            if (ub == 4) {
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    ubuf[q] = idx + q >= M ? 0.0
                              : upre ? (cg ? __ldcg(upre + idx + q) : upre[idx + q])
                                     : draws.get(cr, chain, step, idx + q);
                ub = 0;
            }
            const double u = ubuf[ub++];
            ++idx;
            if (i == M - 1) {
                const int v = (u < (double)(f0 / (f0 + f1))) ? 0 : 1;
                dmap = v | (v << 1);
            } else {
                const float t = tof(i + 1), a = 1.f - t;
                const float x0 = f0 * a, y0 = f1 * t;   // next = 0
                const float x1 = f0 * t, y1 = f1 * a;   // next = 1
                const int d0 = (u < (double)(x0 / (x0 + y0))) ? 0 : 1;
                const int d1 = (u < (double)(x1 / (x1 + y1))) ? 0 : 1;
                dmap = d0 | (d1 << 1);
            }
        }
        maps[i] = (uint8_t)dmap;
        gmap = map_compose(dmap, gmap);
    }
    // suffix composition x_k = G_k o G_{k+1} o ... o G_{T-1}: within the warp,
    // then across warps
    int xm = gmap;
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_down_sync(FULLMASK, xm, d);
        if (lane + d < 32) xm = map_compose(xm, y);
    }
    if (lane == 0) sc.wmap[warp] = xm;
    __syncthreads();
    if (tid == 0) {
        int acc = 2;
        sc.wmap[nw] = 2;
        for (int w = nw - 1; w >= 0; --w) {
            acc = map_compose(sc.wmap[w], acc);
            sc.wmap[w] = acc;     // warp w's maps composed with every warp above it
        }
    }
    __syncthreads();
    // the state entering this chunk from above: x_{k+1} applied to anything
    // (the chunk holding locus M-1 ends in a constant map)
    const int tail = sc.wmap[warp + 1];
    const int full = map_compose(xm, tail);
    int above_map = __shfl_down_sync(FULLMASK, full, 1);
    if (lane == 31) above_map = tail;
    int sv = above_map & 1;
    for (int i = s1 - 1; i >= s0; --i) {
        sv = (maps[i] >> sv) & 1;
        uint32_t* wp = G + (size_t)i * P.W + (m >> 5);
        const uint32_t w = words ? words[i] : *wp;
        const int cur = (int)((w >> (m & 31)) & 1u);
        if (sv != cur) *wp = w ^ (1u << (m & 31));
    }
}

__global__ void __launch_bounds__(1024, 1) ffbs_scan_kernel(ProblemDev P, uint32_t* dg, int first, int nchain,
                                                         const int32_t* order, int64_t ostride, int step,
                                                         Draws draws, const uint8_t* sel, int want,
                                                         const uint8_t* badc, const float* raw32, float* fbbuf,
                                                         uint8_t* mapbuf, int staged, const double* ubuf) {
    extern __shared__ __align__(16) unsigned char fsm[];
    const int cr = blockIdx.x;
    if (cr >= nchain) return;
    if (sel && sel[cr] != want) return;
    if (badc[cr]) return;
    const int M = P.M;
    ffbs_scan_chain(P, dg, first + cr, cr, order[cr * ostride + step], step, draws,
                    ubuf ? ubuf + (size_t)cr * M : nullptr,
                    raw32 + (size_t)cr * 2 * M, fbbuf + (size_t)cr * 2 * M, mapbuf + (size_t)cr * M, staged, false,
                    fsm);
}

// ---------------------------------------------------------------------------
// Fast M-sampler likelihoods of one meiosis step: grid (blocks per chain,
// chains), one warp per locus (fagw_task).  With ubuf, the first 32-locus
// slice of warps also draws the step's uniforms by index, one per lane, so
// ffbs_scan_kernel only reads them.
// ---------------------------------------------------------------------------
template <int G, typename E>
__global__ void __launch_bounds__(kFagWarpsPerBlock * 32) fag_warp_kernel(ProblemDev P, uint32_t* dg, int first,
                                                                         const int32_t* order, int64_t ostride,
                                                                         int step, Draws draws, const uint8_t* sel,
                                                                         int want, float* rawbuf, float* raw32,
                                                                         uint8_t* badc, int* status, double* ubuf) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int cr = blockIdx.y;
    if (sel && sel[cr] != want) return;
    const int M = P.M;
    const FagwTables tab = fagw_load_tables(P, smem);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kLoci = 32 / G;   // loci per warp
    const int chain = first + cr;
    const int32_t* ord = order + cr * ostride;
    const int gw = blockIdx.x * kFagWarpsPerBlock + warp;
    if (ubuf && step >= 0 && gw * 32 + lane < M)
        ubuf[(size_t)cr * M + gw * 32 + lane] = draws.get(cr, chain, step, gw * 32 + lane);
    const int gi = lane / G, l = gw * kLoci + gi;
    if (gw * kLoci < M)
        fagw_task<G, E>(P, tab,
                        smem + fagw_tables(P.N) + ((size_t)warp * kLoci + gi) * fagw_warp_bytes(P.N, P.F, (int)sizeof(E)),
                        dg, chain,
                     cr, l, l < M, ord, step, rawbuf, raw32, badc, status);
}

// Threads per chain of ffbs_scan_kernel: runs of about 2 loci (the scan is
// on every meiosis step's critical path; shorter runs shorten its serial parts).
int ffbs_scan_threads(int M) {
    int t = ((M + 1) / 2 + 31) / 32 * 32;
    return t < 32 ? 32 : (t > 1024 ? 1024 : t);
}

// Shared bytes: the scan scratch, then (when staged) the chain's arrays.
size_t ffbs_scan_scratch(int T) { return (size_t)16 * T + 16 * 32 + 4 * 32 + 4 * 36; }
size_t ffbs_scan_smem(int M) { return ffbs_scan_scratch(ffbs_scan_threads(M)) + (size_t)6 * 4 * M + (size_t)M + 16; }

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
                    if constexpr (sizeof(T) == 8) {
                        const int e = ilogb(mx);
                        const T f = scalbn(1.0, -e);
                        for (int cell = lane; cell < ncell; cell += 32) out[cell] *= f;
                        scale += e;
                    } else {
                        // FP32: the largest cell to 2^scale_to (LI_SCALE, sl_internal.h)
                        const int e = ilogbf(mx) - op.scale_to;
                        for (int cell = lane; cell < ncell; cell += 32) out[cell] = ldexpf(out[cell], -e);
                        scale += e;
                    }
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
                if (!P.lod_zero_ok) set_status(status, ST_LOD_NONPOS);
                v = -DBL_MAX;
            } else {
                v = log(r) + (double)scale * 0.69314718055994530942 - rec - P.marker_trans;
            }
            vals[t] = v;
        }
        __syncwarp();
    }
}

// Batched trait peel: one thread per (graph, interval, position) runs the
// compiled LI_* program; every lane of a warp executes the same instruction
// stream (uniform loads of the program) on its own recombination terms, with
// its FP32 slots in shared memory at [slot][thread].  Each rfunction's cells
// are rescaled by a power of two after they are computed; the exponents are
// summed and restored in FP64 at the end.
__global__ void __launch_bounds__(128) lod_prog_kernel(ProblemDev P, const uint32_t* graphs, int64_t graph_words,
                                                       int G, double* vals, int* status) {
    extern __shared__ float sh[];
    const int S = blockDim.x;
    float* A = sh + threadIdx.x;
    const int n = P.n_lod;
    const int64_t npos = (int64_t)(P.M - 1) * n;
    const int64_t ntask = (int64_t)G * npos;
    for (int64_t t = (int64_t)blockIdx.x * S + threadIdx.x; t < ntask; t += (int64_t)gridDim.x * S) {
        const int b = (int)(t / npos);
        const int64_t pidx = t % npos;
        const int l = (int)(pidx / n), o = (int)(pidx % n);
        const uint32_t* colL = graphs + (size_t)b * graph_words + (size_t)l * P.W;
        const uint32_t* colR = colL + P.W;
        const float th = P.partial_f[l] * (float)(o + 1), an = 1.f - th;
        const float th2 = P.partial_f[l] * (float)(n - o), an2 = 1.f - th2;
        int scale = 0;
        float result = 0.f;
        const int32_t* pc = P.prog;
        while (true) {
            const int op = __ldg(pc);
            if (op == LI_CELL) {
                const int dst = __ldg(pc + 1), nt = __ldg(pc + 2);
                pc += 3;
                float total = 0.f;
                for (int q = 0; q < nt; ++q) {
                    const int nf = __ldg(pc);
                    float v = __ldg(P.pconst + __ldg(pc + 1));
                    pc += 2;
                    for (int f = 0; f < nf; ++f) v *= A[__ldg(pc + f) * S];
                    pc += nf;
                    total += v;
                }
                A[dst * S] = total;
            } else if (op == LI_REC) {
                const int child = __ldg(pc + 1), dst = __ldg(pc + 2);
                pc += 3;
                const int bits = person_bits(P, colL, colR, child);
                A[(dst + 0) * S] = 0.25f * trait_rec<float>(bits, 0, 0, th, an, th2, an2);
                A[(dst + 1) * S] = 0.25f * trait_rec<float>(bits, 0, 1, th, an, th2, an2);
                A[(dst + 2) * S] = 0.25f * trait_rec<float>(bits, 1, 0, th, an, th2, an2);
                A[(dst + 3) * S] = 0.25f * trait_rec<float>(bits, 1, 1, th, an, th2, an2);
            } else if (op == LI_SUM) {
                const int dst = __ldg(pc + 1), ns = __ldg(pc + 2);
                float v = 0.f;
                for (int q = 0; q < ns; ++q) v += A[__ldg(pc + 3 + q) * S];
                A[dst * S] = v;
                pc += 3 + ns;
            } else if (op == LI_SCALE) {
                const int first = __ldg(pc + 1), cnt = __ldg(pc + 2), target = __ldg(pc + 3);
                pc += 4;
                float mx = 0.f;
                for (int q = 0; q < cnt; ++q) mx = fmaxf(mx, A[(first + q) * S]);
                if (mx > 0.f) {
                    // ldexpf: exact for any exponent, a subnormal maximum included
                    const int e = ilogbf(mx) - target;
                    for (int q = 0; q < cnt; ++q) A[(first + q) * S] = ldexpf(A[(first + q) * S], -e);
                    scale += e;
                }
            } else {
                const int rs = __ldg(pc + 1);
                result = rs >= 0 ? A[rs * S] : 0.f;
                break;
            }
        }
        // DescentGraph::get_recombination_prob (descent_graph.cc:212-242) by crossover count
        int cross = 0;
        for (int w = 0; w < P.W; ++w) cross += __popc(colL[w] ^ colR[w]);
        const double rec = cross * P.log_theta[l] + (2 * P.Nnf - cross) * P.log_itheta[l];
        double v;
        if (!(result > 0.f)) {
            if (!P.lod_zero_ok) set_status(status, ST_LOD_NONPOS);
            v = -DBL_MAX;
        } else {
            // log of an FP32 value in FP32 (error ~1e-7, far inside the LOD tolerance)
            v = (double)logf(result) + (double)scale * 0.69314718055994530942 - rec - P.marker_trans;
        }
        vals[t] = v;
    }
}

// Adjoint of the trait peel (the reverse sum-product of TraitRfunction's
// peel, trait_rfunction.cc:28-137), one warp per (graph, interval, position)
// task with the rfunctions in the warp's shared memory, dense [4^c] per op
// (every cell and term kept: a zero disease probability still has a
// derivative with respect to the model).
//
// Forward: as the FP32 scorer, one (cell, term) item per lane -- a child
// peel's terms are its four transmissions (i, j), the others' the peel node's
// four states -- each rfunction scaled so its largest cell is 2^scale_to, the
// exponent kept.  Reverse: B[root] = 1 / root; op k's cell adjoint times
// 2^-e_k (its scaling) is spread over the item's factors: to each previous
// rfunction's cell (shared-memory atomics: cells of op k that differ only in
// members outside that cutset meet there), to the peel node's disease
// probability (its derivatives by the three penetrances and the frequency)
// and, through the children's recombination terms, to theta_L and theta_R.
// The exponents are constants of the pass, so working on scaled values gives
// d log L exactly.
//
// Memory (AdjDev): with one segment every matrix is kept from the forward
// pass (store).  When that does not fit the per-warp budget the ops are split
// into segments: the first forward pass keeps only matrices a later segment
// reads, and before each earlier segment's reverse pass its other matrices
// are recomputed from the kept ones (recompute instead of store; one extra
// forward pass).  graphs == nullptr peels without a graph (every
// recombination term 1/4, Peeler::calc_trait_prob): one task, no theta
// derivatives.  grad[task - task0][6] = d log L / d (theta_L, theta_R,
// pen x3, frequency), FP64.
constexpr int kAdjMaxPrev = 8;

struct AdjTask {
    const uint32_t* colL;
    const uint32_t* colR;
    float th, an, th2, an2;
    bool graph;
};

// 0.25 x the recombination term of (i, j) and its derivatives by theta_L and
// theta_R (TraitRfunction::get_recombination_probability, trait_rfunction.cc:9-24)
__device__ __forceinline__ void adj_rec(const AdjTask& T, int bits, int i, int j, float& r, float& dl, float& dr) {
    if (!T.graph) {
        r = 0.25f;
        dl = dr = 0.f;
        return;
    }
    const bool ml = (bits & 1) == i, mr = ((bits >> 2) & 1) == i;
    const bool pl = ((bits >> 1) & 1) == j, pr = ((bits >> 3) & 1) == j;
    const float x0 = ml ? T.an : T.th, x1 = mr ? T.an2 : T.th2, x2 = pl ? T.an : T.th, x3 = pr ? T.an2 : T.th2;
    const float s0 = ml ? -1.f : 1.f, s1 = mr ? -1.f : 1.f, s2 = pl ? -1.f : 1.f, s3 = pr ? -1.f : 1.f;
    r = 0.25f * (x0 * x1 * x2 * x3);
    dl = 0.25f * (s0 * x1 * x2 * x3 + x0 * x1 * s2 * x3);
    dr = 0.25f * (x0 * s1 * x2 * x3 + x0 * x1 * x2 * s3);
}

// Op k's recombination terms at this task, for a child peel its child's and
// for a parent peel each child's: for (i, j) = 2i + j, 0.25 x the term and its
// derivatives by theta_L and theta_R at rt[12 c + b], rt[12 c + 4 + b],
// rt[12 c + 8 + b] (the warp's scratch; its items read them).
__device__ __forceinline__ void adj_rtab(const ProblemDev& P, const AdjTask& T, const OpDev& op, float* rt, int lane) {
    const int nch = op.type == CHILD ? 1 : (op.type == PARENT ? op.n_child : 0);
    for (int q = lane; q < 4 * nch; q += 32) {
        const int c = q >> 2, b = q & 3;
        const int child = op.type == CHILD ? op.peel : P.opdata[op.child_at + 4 * c];
        const int bits = T.graph ? person_bits(P, T.colL, T.colR, child) : 0;
        float r, dl, dr;
        adj_rec(T, bits, b >> 1, b & 1, r, dl, dr);
        rt[12 * c + b] = r;
        rt[12 * c + 4 + b] = dl;
        rt[12 * c + 8 + b] = dr;
    }
    __syncwarp();
}

// Child c's transmission mask of an item of a parent peel (AdjDev::items).
__device__ __forceinline__ uint32_t adj_mask(const uint32_t* w, int pw, int c) {
    return c < 7 ? (w[0] >> (2 + 4 * c)) & 15u : (w[1 + pw + (c - 7) / 8] >> (4 * ((c - 7) % 8))) & 15u;
}

// The item's product of recombination factors (and, with D, its derivatives
// by theta_L and theta_R by the product rule as it is built): a child peel's
// one term, a parent peel's per-child sums of the transmissions its mask
// lets through, in transmission order.
template <bool D>
__device__ __forceinline__ void adj_R(const OpDev& op, const uint32_t* w, int pw, int t, const float* rt, float& R,
                                      float& dRl, float& dRr) {
    R = 1.f;
    dRl = dRr = 0.f;
    if (op.type == CHILD) {
        R = rt[t];
        if (D) {
            dRl = rt[4 + t];
            dRr = rt[8 + t];
        }
    } else if (op.type == PARENT) {
        for (int c = 0; c < op.n_child; ++c) {
            const uint32_t mask = adj_mask(w, pw, c);
            float sc = 0.f, sl = 0.f, sr = 0.f;
#pragma unroll
            for (int b = 0; b < 4; ++b)
                if (mask & (1u << b)) {
                    sc += rt[12 * c + b];
                    if (D) {
                        sl += rt[12 * c + 4 + b];
                        sr += rt[12 * c + 8 + b];
                    }
                }
            if (D) {
                dRl = dRl * sc + R * sl;
                dRr = dRr * sc + R * sr;
            }
            R *= sc;
        }
    }
}

// 2^-e as a float multiplier when it is a normal number (the op's scaling,
// exact), else 0 (the caller then scales with ldexpf).
__device__ __forceinline__ float adj_pow2(int e) {
    return (e >= -127 && e <= 126) ? __int_as_float((127 - e) << 23) : 0.f;
}

// Forward of op k: its scaled matrix in A, its exponent in E[k].  One item
// per lane: the peel node's disease probability times the previous
// rfunctions' cells times the recombination factors; the four items of a
// cell added by shuffles.
__device__ void adj_forward(const ProblemDev& P, const AdjDev& D, const AdjTask& T, int k, float* A, int* E, float* rt,
                            int lane) {
    const OpDev op = P.ops[k];
    adj_rtab(P, T, op, rt, lane);
    const int ncell = 1 << (2 * op.c), nitem = 4 * ncell;
    const int nw = adj_item_words(op.n_prev, op.n_child), pw = (op.n_prev + 1) / 2;
    const uint32_t* tab = D.items + D.item_at[k];
    float* out = A + D.aoff[k];
    const float* dp = D.dprob + 4 * op.peel;
    float mx = 0.f;
    for (int it0 = 0; it0 < nitem; it0 += 32) {
        const int item = it0 + lane, cell = item >> 2, t = item & 3;
        float term = 0.f;
        if (item < nitem) {
            const uint32_t* w = tab + (size_t)item * nw;
            term = dp[w[0] & 3u];
            for (int j = 0; j < op.n_prev; ++j) term *= A[(w[1 + (j >> 1)] >> (16 * (j & 1))) & 0xffffu];
            float R, dl, dr;
            adj_R<false>(op, w, pw, t, rt, R, dl, dr);
            term *= R;
        }
        const int grp = lane & ~3;
        const float t0 = __shfl_sync(FULLMASK, term, grp), t1 = __shfl_sync(FULLMASK, term, grp + 1);
        const float t2 = __shfl_sync(FULLMASK, term, grp + 2), t3 = __shfl_sync(FULLMASK, term, grp + 3);
        if (t == 0 && item < nitem) {
            const float total = ((t0 + t1) + t2) + t3;
            out[cell] = total;
            mx = fmaxf(mx, total);
        }
    }
    for (int dd = 16; dd >= 1; dd >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULLMASK, mx, dd));
    const int e = mx > 0.f ? ilogbf(mx) - op.scale_to : 0;
    const float sc = adj_pow2(e);
    __syncwarp();
    for (int cell = lane; cell < ncell; cell += 32) out[cell] = sc != 0.f ? out[cell] * sc : ldexpf(out[cell], -e);
    if (lane == 0) E[k] = e;
    __syncwarp();
}

// The items of op k in the reverse pass, NP previous rfunctions (unrolled).
template <int NP>
__device__ __forceinline__ void adj_reverse_items(const OpDev& op, const uint32_t* tab, int nw, int pw, int nitem,
                                                  const float* bk, int e, const float* A, float* B, const float* dp,
                                                  const float4* dg, const float* rt, int lane, float* acc) {
    const float sc = adj_pow2(e);
    float gl = 0.f, gr = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;
    for (int it0 = 0; it0 < nitem; it0 += 32) {
        const int item = it0 + lane, cell = item >> 2, t = item & 3;
        if (item >= nitem) break;
        const float gd = sc != 0.f ? bk[cell] * sc : ldexpf(bk[cell], -e);   // the cell's adjoint before its scaling
        if (gd == 0.f) continue;
        const uint32_t* w = tab + (size_t)item * nw;
        const int s = (int)(w[0] & 3u);
        float a[NP > 0 ? NP : 1];
        int off[NP > 0 ? NP : 1];
        float pp = 1.f;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
            off[j] = (int)((w[1 + (j >> 1)] >> (16 * (j & 1))) & 0xffffu);
            a[j] = A[off[j]];
            pp *= a[j];
        }
        float R, dRl, dRr;
        adj_R<true>(op, w, pw, t, rt, R, dRl, dRr);
        const float c = dp[s];
        const float wgt = gd * pp;
        const float4 dc = dg[s];
        g0 += wgt * R * dc.x;
        g1 += wgt * R * dc.y;
        g2 += wgt * R * dc.z;
        g3 += wgt * R * dc.w;
        gl += wgt * c * dRl;
        gr += wgt * c * dRr;
        // each factor's adjoint: the product of the others, by prefix and suffix products
        float pre[NP > 0 ? NP : 1];
        float run = gd * c * R;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
            pre[j] = run;
            run *= a[j];
        }
        float suf = 1.f;
#pragma unroll
        for (int j = NP - 1; j >= 0; --j) {
            const float v = pre[j] * suf;
            if (v != 0.f) atomicAdd(B + off[j], v);
            suf *= a[j];
        }
    }
    acc[0] += gl;
    acc[1] += gr;
    acc[2] += g0;
    acc[3] += g1;
    acc[4] += g2;
    acc[5] += g3;
}

// Reverse of op k: adjoints into the previous rfunctions' cells (B), the
// model derivatives into g.
__device__ void adj_reverse(const ProblemDev& P, const AdjDev& D, const AdjTask& T, int k, const float* A, float* B,
                            const int* E, float* rt, int lane, double* g) {
    const OpDev op = P.ops[k];
    adj_rtab(P, T, op, rt, lane);
    const int ncell = 1 << (2 * op.c), nitem = 4 * ncell;
    const int nw = adj_item_words(op.n_prev, op.n_child), pw = (op.n_prev + 1) / 2;
    const uint32_t* tab = D.items + D.item_at[k];
    const float* bk = B + D.aoff[k];
    const float* dp = D.dprob + 4 * op.peel;
    const float4* dg = D.dgrad + 4 * op.peel;
    const int e = E[k];
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    switch (op.n_prev) {
#define SL_ADJ_NP(n) \
        case n: adj_reverse_items<n>(op, tab, nw, pw, nitem, bk, e, A, B, dp, dg, rt, lane, acc); break;
        SL_ADJ_NP(0) SL_ADJ_NP(1) SL_ADJ_NP(2) SL_ADJ_NP(3) SL_ADJ_NP(4)
        SL_ADJ_NP(5) SL_ADJ_NP(6) SL_ADJ_NP(7) SL_ADJ_NP(8)
#undef SL_ADJ_NP
        default: break;
    }
    for (int q = 0; q < 6; ++q) g[q] += (double)acc[q];
    __syncwarp();
}

__global__ void __launch_bounds__(128) trait_adjoint_kernel(ProblemDev P, AdjDev D, const uint32_t* graphs,
                                                            int64_t graph_words, int64_t task0, int64_t ntask,
                                                            double* grad, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* A = (float*)(smem + (size_t)warp * D.warp_bytes);
    float* B = A + D.half;
    int* E = (int*)(B + D.half);
    float* rt = (float*)(E + P.K);   // [12 max_child] the op's recombination terms
    const int n = P.n_lod;
    const int64_t npos = (int64_t)(P.M - 1) * n;
    for (int64_t u = (int64_t)blockIdx.x * wpb + warp; u < ntask; u += (int64_t)gridDim.x * wpb) {
        const int64_t t = task0 + u;
        AdjTask T;
        T.graph = graphs != nullptr;
        T.colL = T.colR = nullptr;
        T.th = T.an = T.th2 = T.an2 = 0.f;
        if (T.graph) {
            const int b = (int)(t / npos);
            const int64_t pidx = t % npos;
            const int l = (int)(pidx / n), o = (int)(pidx % n);
            T.colL = graphs + (size_t)b * graph_words + (size_t)l * P.W;
            T.colR = T.colL + P.W;
            T.th = P.partial_f[l] * (float)(o + 1);
            T.an = 1.f - T.th;
            T.th2 = P.partial_f[l] * (float)(n - o);
            T.an2 = 1.f - T.th2;
        }
        // first forward pass: every op; matrices not kept are overwritten by later segments
        for (int k = 0; k < P.K; ++k) adj_forward(P, D, T, k, A, E, rt, lane);
        const float root = A[D.aoff[P.K - 1]];
        double g[6] = {0, 0, 0, 0, 0, 0};
        if (!(root > 0.f)) {
            if (lane == 0) {
                if (!P.lod_zero_ok) set_status(status, ST_LOD_NONPOS);
                for (int q = 0; q < 6; ++q) grad[u * 6 + q] = __longlong_as_double(0x7ff8000000000000LL);   // NaN
            }
            __syncwarp();
            continue;
        }
        for (int i = lane; i < D.half; i += 32) B[i] = 0.f;
        __syncwarp();
        for (int sg = D.nseg - 1; sg >= 0; --sg) {
            const int k0 = D.seg[sg], k1 = D.seg[sg + 1];
            if (sg < D.nseg - 1) {
                // recompute the segment's matrices that were not kept, zero their adjoints
                for (int k = k0; k < k1; ++k)
                    if (!D.keep[k]) adj_forward(P, D, T, k, A, E, rt, lane);
                for (int k = k0; k < k1; ++k)
                    if (!D.keep[k])
                        for (int i = lane; i < (1 << (2 * P.ops[k].c)); i += 32) B[D.aoff[k] + i] = 0.f;
                __syncwarp();
            } else if (lane == 0) {
                B[D.aoff[P.K - 1]] = 1.0f / root;
            }
            __syncwarp();
            for (int k = k1 - 1; k >= k0; --k) adj_reverse(P, D, T, k, A, B, E, rt, lane, g);
        }
        for (int q = 0; q < 6; ++q) {
            double v = g[q];
            for (int dd = 16; dd >= 1; dd >>= 1) v += __shfl_xor_sync(FULLMASK, v, dd);
            if (lane == 0) grad[u * 6 + q] = v;
        }
        __syncwarp();
    }
}

// The same adjoint with one thread per task: each thread's matrices and
// adjoints live in global memory, a column of the arena per resident thread
// (float offset o of thread r at o * nthr + r, so the threads of a warp, all
// at the same item, touch one 128-byte line), and every item of an op is the
// thread's own serial loop, so small rfunctions leave no lane idle and the
// adjoints need no atomics.  Matrices are stored unscaled with their
// exponents; a factor is scaled as it is read, which gives the scaled form's
// values exactly.  Same plan (offsets, segments, kept matrices) and item
// tables as the warp form.
struct AdjThr {
    float* A;       // arena base of this thread: A[o * nthr]
    float* B;       // adjoints: B[o * nthr]
    int* E;         // exponents: E[k * nthr]
    int64_t nthr;
};

// The thread's recombination terms of op k, rt[12 c + b] as in adj_rtab.
__device__ __forceinline__ void adj_rtab_thr(const ProblemDev& P, const AdjTask& T, const OpDev& op, float* rt) {
    const int nch = op.type == CHILD ? 1 : (op.type == PARENT ? op.n_child : 0);
    for (int c = 0; c < nch; ++c) {
        const int child = op.type == CHILD ? op.peel : P.opdata[op.child_at + 4 * c];
        const int bits = T.graph ? person_bits(P, T.colL, T.colR, child) : 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            float r, dl, dr;
            adj_rec(T, bits, b >> 1, b & 1, r, dl, dr);
            rt[12 * c + b] = r;
            rt[12 * c + 4 + b] = dl;
            rt[12 * c + 8 + b] = dr;
        }
    }
}

// Factor j's scale and exponent for op k's previous rfunctions.
__device__ __forceinline__ void adj_prev_scales(const ProblemDev& P, const AdjThr& R, const OpDev& op, float* sj,
                                                int* ej) {
    const int32_t* po = P.opdata + op.prev_ops_at;
    for (int j = 0; j < op.n_prev; ++j) {
        ej[j] = R.E[(int64_t)po[j] * R.nthr];
        sj[j] = adj_pow2(ej[j]);
    }
}

__device__ __forceinline__ float adj_scaled(float v, float sc, int e) { return sc != 0.f ? v * sc : ldexpf(v, -e); }

__device__ void adj_forward_thr(const ProblemDev& P, const AdjDev& D, const AdjTask& T, const AdjThr& R, int k,
                                float* rt) {
    const OpDev op = P.ops[k];
    adj_rtab_thr(P, T, op, rt);
    float sj[kAdjMaxPrev];
    int ej[kAdjMaxPrev];
    adj_prev_scales(P, R, op, sj, ej);
    const int ncell = 1 << (2 * op.c);
    const int nw = adj_item_words(op.n_prev, op.n_child), pw = (op.n_prev + 1) / 2;
    const uint32_t* tab = D.items + D.item_at[k];
    float* out = R.A + (int64_t)D.aoff[k] * R.nthr;
    const float* dp = D.dprob + 4 * op.peel;
    float mx = 0.f;
    for (int cell = 0; cell < ncell; ++cell) {
        float tv[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const uint32_t* w = tab + (size_t)(4 * cell + t) * nw;
            float term = dp[w[0] & 3u];
            for (int j = 0; j < op.n_prev; ++j) {
                const int off = (int)((w[1 + (j >> 1)] >> (16 * (j & 1))) & 0xffffu);
                term *= adj_scaled(R.A[(int64_t)off * R.nthr], sj[j], ej[j]);
            }
            float Rr, dl, dr;
            adj_R<false>(op, w, pw, t, rt, Rr, dl, dr);
            tv[t] = term * Rr;
        }
        const float total = ((tv[0] + tv[1]) + tv[2]) + tv[3];
        out[(int64_t)cell * R.nthr] = total;
        mx = fmaxf(mx, total);
    }
    R.E[(int64_t)k * R.nthr] = mx > 0.f ? ilogbf(mx) - op.scale_to : 0;
}

template <int NP>
__device__ __forceinline__ void adj_reverse_thr_items(const OpDev& op, const uint32_t* tab, int nw, int pw, int ncell,
                                                      const AdjThr& R, const float* bk, float sk, int ek,
                                                      const float* sj, const int* ej, const float* dp,
                                                      const float4* dg, const float* rt, float* acc) {
    float gl = 0.f, gr = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f, g3 = 0.f;
    for (int cell = 0; cell < ncell; ++cell) {
        const float gd = adj_scaled(bk[(int64_t)cell * R.nthr], sk, ek);   // the cell's adjoint before its scaling
        if (gd == 0.f) continue;
#pragma unroll 1
        for (int t = 0; t < 4; ++t) {
            const uint32_t* w = tab + (size_t)(4 * cell + t) * nw;
            const int s = (int)(w[0] & 3u);
            float a[NP > 0 ? NP : 1];
            int off[NP > 0 ? NP : 1];
            float pp = 1.f;
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                off[j] = (int)((w[1 + (j >> 1)] >> (16 * (j & 1))) & 0xffffu);
                a[j] = adj_scaled(R.A[(int64_t)off[j] * R.nthr], sj[j], ej[j]);
                pp *= a[j];
            }
            float Rr, dRl, dRr;
            adj_R<true>(op, w, pw, t, rt, Rr, dRl, dRr);
            const float c = dp[s];
            const float wgt = gd * pp;
            const float4 dc = dg[s];
            g0 += wgt * Rr * dc.x;
            g1 += wgt * Rr * dc.y;
            g2 += wgt * Rr * dc.z;
            g3 += wgt * Rr * dc.w;
            gl += wgt * c * dRl;
            gr += wgt * c * dRr;
            float pre[NP > 0 ? NP : 1];
            float run = gd * c * Rr;
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                pre[j] = run;
                run *= a[j];
            }
            float suf = 1.f;
#pragma unroll
            for (int j = NP - 1; j >= 0; --j) {
                const float v = pre[j] * suf;
                if (v != 0.f) R.B[(int64_t)off[j] * R.nthr] += v;
                suf *= a[j];
            }
        }
    }
    acc[0] += gl;
    acc[1] += gr;
    acc[2] += g0;
    acc[3] += g1;
    acc[4] += g2;
    acc[5] += g3;
}

__device__ void adj_reverse_thr(const ProblemDev& P, const AdjDev& D, const AdjTask& T, const AdjThr& R, int k,
                                float* rt, double* g) {
    const OpDev op = P.ops[k];
    adj_rtab_thr(P, T, op, rt);
    float sj[kAdjMaxPrev];
    int ej[kAdjMaxPrev];
    adj_prev_scales(P, R, op, sj, ej);
    const int ncell = 1 << (2 * op.c);
    const int nw = adj_item_words(op.n_prev, op.n_child), pw = (op.n_prev + 1) / 2;
    const uint32_t* tab = D.items + D.item_at[k];
    const float* bk = R.B + (int64_t)D.aoff[k] * R.nthr;
    const int ek = R.E[(int64_t)k * R.nthr];
    const float sk = adj_pow2(ek);
    const float* dp = D.dprob + 4 * op.peel;
    const float4* dg = D.dgrad + 4 * op.peel;
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    switch (op.n_prev) {
#define SL_ADJ_NP(n) \
        case n: adj_reverse_thr_items<n>(op, tab, nw, pw, ncell, R, bk, sk, ek, sj, ej, dp, dg, rt, acc); break;
        SL_ADJ_NP(0) SL_ADJ_NP(1) SL_ADJ_NP(2) SL_ADJ_NP(3) SL_ADJ_NP(4)
        SL_ADJ_NP(5) SL_ADJ_NP(6) SL_ADJ_NP(7) SL_ADJ_NP(8)
#undef SL_ADJ_NP
        default: break;
    }
    for (int q = 0; q < 6; ++q) g[q] += (double)acc[q];
}

__global__ void __launch_bounds__(128, 6) trait_adjoint_thr_kernel(ProblemDev P, AdjDev D, const uint32_t* graphs,
                                                                int64_t graph_words, int64_t task0, int64_t ntask,
                                                                double* grad, int* status, float* arena, int* expo) {
    const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    AdjThr R;
    R.nthr = nthr;
    R.A = arena + r;
    R.B = arena + (int64_t)D.half * nthr + r;
    R.E = expo + r;
    float rt[12 * 32];   // the op's recombination terms (local memory)
    const int n = P.n_lod;
    const int64_t npos = (int64_t)(P.M - 1) * n;
    for (int64_t u = r; u < ntask; u += nthr) {
        const int64_t t = task0 + u;
        AdjTask T;
        T.graph = graphs != nullptr;
        T.colL = T.colR = nullptr;
        T.th = T.an = T.th2 = T.an2 = 0.f;
        if (T.graph) {
            const int b = (int)(t / npos);
            const int64_t pidx = t % npos;
            const int l = (int)(pidx / n), o = (int)(pidx % n);
            T.colL = graphs + (size_t)b * graph_words + (size_t)l * P.W;
            T.colR = T.colL + P.W;
            T.th = P.partial_f[l] * (float)(o + 1);
            T.an = 1.f - T.th;
            T.th2 = P.partial_f[l] * (float)(n - o);
            T.an2 = 1.f - T.th2;
        }
        for (int k = 0; k < P.K; ++k) adj_forward_thr(P, D, T, R, k, rt);
        const int kr = P.K - 1;
        const int er = R.E[(int64_t)kr * nthr];
        const float root = adj_scaled(R.A[(int64_t)D.aoff[kr] * nthr], adj_pow2(er), er);
        double g[6] = {0, 0, 0, 0, 0, 0};
        if (!(root > 0.f)) {
            if (!P.lod_zero_ok) set_status(status, ST_LOD_NONPOS);
            for (int q = 0; q < 6; ++q) grad[u * 6 + q] = __longlong_as_double(0x7ff8000000000000LL);   // NaN
            continue;
        }
        for (int i = 0; i < D.half; ++i) R.B[(int64_t)i * nthr] = 0.f;
        for (int sg = D.nseg - 1; sg >= 0; --sg) {
            const int k0 = D.seg[sg], k1 = D.seg[sg + 1];
            if (sg < D.nseg - 1) {
                // recompute the segment's matrices that were not kept, zero their adjoints
                for (int k = k0; k < k1; ++k)
                    if (!D.keep[k]) adj_forward_thr(P, D, T, R, k, rt);
                for (int k = k0; k < k1; ++k)
                    if (!D.keep[k])
                        for (int i = 0; i < (1 << (2 * P.ops[k].c)); ++i) R.B[(int64_t)(D.aoff[k] + i) * nthr] = 0.f;
            } else {
                R.B[(int64_t)D.aoff[kr] * nthr] = 1.0f / root;
            }
            for (int k = k1 - 1; k >= k0; --k) adj_reverse_thr(P, D, T, R, k, rt, g);
        }
        for (int q = 0; q < 6; ++q) grad[u * 6 + q] = g[q];
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
        uint8_t ini = init ? init[p] : 1;   // without flags, acc starts at -DBL_MAX
        for (int b = 0; b < G; ++b) {
            const double v = vals[(size_t)b * npos + p];
            a = ini ? log_sum(v, a) : v;
            ini = 1;
        }
        acc[p] = a;
        if (init) init[p] = ini;
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
// Parts of log P(G, graph) under a chain's map (DescentGraph::get_likelihood,
// descent_graph.cc:184-269), for up to four (graph chain, map chain) pairs:
// the founder-allele-graph likelihood of every locus (exact FP64, as the
// M-sampler's) and the recombination log-probability of every interval, each
// a sum in the reference's order; the host adds them up in order.
// ---------------------------------------------------------------------------
template <typename IX>
__global__ void __launch_bounds__(128) loglik_fag_kernel(ProblemDev P, const uint32_t* dg, int4 gch, int4 tch,
                                                         int npair, double* out, const Mc3Dev* m) {
    if (m) {   // the pairs of the device-side exchange, if one is due
        if (!m->active) return;
        gch = make_int4(m->gch[0], m->gch[1], m->gch[2], m->gch[3]);
        tch = make_int4(m->tch[0], m->tch[1], m->tch[2], m->tch[3]);
    }
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = blockDim.x;
    const size_t per = fag_block_bytes(P.N, P.F, S, 0) - (((size_t)P.N * 7 + 15) & ~(size_t)15);
    int16_t* s_order = (int16_t*)(smem + per);
    int16_t* s_mo = s_order + P.N;
    int16_t* s_fa = s_mo + P.N;
    uint8_t* s_typed = (uint8_t*)(s_fa + P.N);
    for (int i = threadIdx.x; i < P.N; i += S) {
        s_order[i] = P.fag_order[i];
        s_mo[i] = P.mother[i];
        s_fa[i] = P.father[i];
        s_typed[i] = P.typed[i];
    }
    __syncthreads();
    Fag<IX, double> fs = fag_bind<IX, double>(smem, P.N, P.F, S, threadIdx.x);
    const int64_t t = (int64_t)blockIdx.x * S + threadIdx.x;
    if (t >= (int64_t)npair * P.M) return;
    const int k = (int)(t / P.M), l = (int)(t % P.M);
    const int g = k == 0 ? gch.x : k == 1 ? gch.y : k == 2 ? gch.z : gch.w;
    const int tc = k == 0 ? tch.x : k == 1 ? tch.y : k == 2 ? tch.z : tch.w;
    const uint32_t* col = dg + ((size_t)g * P.M + l) * P.W;
    fag_edges(P.N, P.F, s_order, s_mo, s_fa, col, fs, -1);
    out[t] = fag_like<ProbExact>(P.N, P.F, s_typed, P.geno + (size_t)l * P.N, P.c_minor[(size_t)tc * P.M + l], fs);
}

__global__ void loglik_rec_kernel(ProblemDev P, const uint32_t* dg, int4 gch, int4 tch, int npair, double* out,
                                  const Mc3Dev* m) {
    if (m) {
        if (!m->active) return;
        gch = make_int4(m->gch[0], m->gch[1], m->gch[2], m->gch[3]);
        tch = make_int4(m->tch[0], m->tch[1], m->tch[2], m->tch[3]);
    }
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int I = P.M - 1;
    if (t >= (int64_t)npair * I) return;
    const int k = (int)(t / I), l = (int)(t % I);
    const int g = k == 0 ? gch.x : k == 1 ? gch.y : k == 2 ? gch.z : gch.w;
    const int tc = k == 0 ? tch.x : k == 1 ? tch.y : k == 2 ? tch.z : tch.w;
    const uint32_t* colL = dg + ((size_t)g * P.M + l) * P.W;
    const uint32_t* colR = colL + P.W;
    const double lt = P.c_log_theta[(size_t)tc * I + l], la = P.c_log_itheta[(size_t)tc * I + l];
    double r = 0.0;
    for (int b = 0; b < 2 * P.Nnf; ++b) r = DADD(r, dgbit(colL, b) != dgbit(colR, b) ? lt : la);
    out[t] = r;
}

// Exchange two chains' descent graphs.
__global__ void swap_graphs_kernel(uint32_t* dg, size_t words, int a, int b) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t x = dg[(size_t)a * words + i];
        dg[(size_t)a * words + i] = dg[(size_t)b * words + i];
        dg[(size_t)b * words + i] = x;
    }
}

cudaError_t launch_loglik_parts(const ProblemDev& P, const uint32_t* dg, const int* gch, const int* tch, int npair,
                                double* fag_out, double* rec_out, cudaStream_t s, const Mc3Dev* m) {
    const int S = 64;
    const size_t smem = fag_block_bytes(P.N, P.F, S, 0);
    const int wide = 2 * P.F > 255 ? 1 : 0;
    {
        cudaError_t e = ensure_smem(wide ? (const void*)loglik_fag_kernel<uint16_t> : (const void*)loglik_fag_kernel<uint8_t>,
                                    smem);
        if (e != cudaSuccess) return e;
    }
    const int4 g4 = gch ? make_int4(gch[0], gch[1], gch[2], gch[3]) : make_int4(0, 0, 0, 0);
    const int4 t4 = tch ? make_int4(tch[0], tch[1], tch[2], tch[3]) : make_int4(0, 0, 0, 0);
    const int64_t nf = (int64_t)npair * P.M;
    if (wide)
        loglik_fag_kernel<uint16_t><<<(int)((nf + S - 1) / S), S, smem, s>>>(P, dg, g4, t4, npair, fag_out, m);
    else
        loglik_fag_kernel<uint8_t><<<(int)((nf + S - 1) / S), S, smem, s>>>(P, dg, g4, t4, npair, fag_out, m);
    const int64_t nr = (int64_t)npair * (P.M - 1);
    loglik_rec_kernel<<<(int)((nr + 127) / 128), 128, 0, s>>>(P, dg, g4, t4, npair, rec_out, m);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// MC3 exchanges on the device (Mc3::run, mc3.cc:117-158).  After a spurt that
// ends on a multiple of the exchange period, a uniformly chosen adjacent pair
// (r, r + 1) swaps graphs with probability min(1, exp((xy + yx) - (xx + yy))),
// the four log-likelihoods of DescentGraph::get_likelihood2 (descent_graph.cc:
// 184-269).  Both uniforms come from the Philox stream: stage 9, counter high
// word (0x3ff << 40) ^ (spurt end << 4), draws 0 and 1.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mc3_hi(int64_t it_end) {
    return (0x3ffull << 40) ^ ((uint64_t)it_end << 4) ^ 9u;
}

// The proposal after the spurt ending at it_end (rp->end when rp is given;
// one thread).
__global__ void mc3_pick_kernel(Mc3Dev* m, const RunParams* rp, int64_t it_end, int C) {
    if (rp) it_end = rp->end;
    m->it_end = it_end;
    m->active = (C >= 2 && m->period > 0 && it_end % m->period == 0) ? 1 : 0;
    if (!m->active) return;
    int r = (int)((C - 1) * philox_u01(m->seed, mc3_hi(it_end), 0));
    if (r > C - 2) r = C - 2;
    m->r = r;
    const int g[4] = {r, r + 1, r + 1, r}, t[4] = {r, r + 1, r, r + 1};   // xx, yy, xy, yx
    for (int k = 0; k < 4; ++k) {
        m->gch[k] = g[k];
        m->tch[k] = t[k];
    }
}

// The decision (one block of 256): each pair's log-likelihood from its parts
// in the reference's order -- the interval log-probabilities added from 0.0,
// marker transmission first, then the log of every locus's founder-allele-graph
// likelihood (LOG_ZERO = -DBL_MAX for an illegal graph), joined by log_product
// (descent_graph.cc:184-269, logarithms.cc:27-29) -- the acceptance, the swap
// and the counts.  The logs are taken in parallel (in place); one thread per
// pair then sums in order.
__global__ void __launch_bounds__(256) mc3_decide_kernel(Mc3Dev* m, int M, double marker_trans, double* fag,
                                                         const double* rec, uint32_t* dg, size_t words,
                                                         int64_t* accept, int64_t* propose) {
    __shared__ int s_zero[4];
    __shared__ double s_ll[4];
    __shared__ int s_acc;
    if (!m->active) return;
    const int tid = threadIdx.x;
    if (tid < 4) s_zero[tid] = 0;
    __syncthreads();
    for (int i = tid; i < 4 * M; i += 256) {
        const double f = fag[i];
        if (f == 0.0) atomicOr(&s_zero[i / M], 1);
        else fag[i] = log(f);
    }
    __syncthreads();
    if (tid < 4) {
        const double LOG_ZERO = -DBL_MAX;
        double r = 0.0;
        const double* rk = rec + (size_t)tid * (M - 1);
        for (int l = 0; l < M - 1; ++l) r += rk[l];
        const double trans = marker_trans + r;
        double prior = 0.0;
        if (s_zero[tid]) {
            prior = LOG_ZERO;
        } else {
            const double* fk = fag + (size_t)tid * M;
            for (int l = 0; l < M; ++l) prior += fk[l];
        }
        s_ll[tid] = (trans == LOG_ZERO || prior == LOG_ZERO) ? LOG_ZERO : trans + prior;
    }
    __syncthreads();
    if (tid == 0) {
        const double ratio = (s_ll[2] + s_ll[3]) - (s_ll[0] + s_ll[1]);
        const double u = philox_u01(m->seed, mc3_hi(m->it_end), 1);
        const int r = m->r;
        propose[r] += 1;
        s_acc = (u == 0.0 || log(u) < fmin(0.0, ratio)) ? 1 : 0;
        if (s_acc) accept[r] += 1;
    }
    __syncthreads();
    if (s_acc) {
        uint32_t* a = dg + (size_t)m->r * words;
        uint32_t* b = a + words;
        for (size_t i = tid; i < words; i += 256) {
            const uint32_t x = a[i];
            a[i] = b[i];
            b[i] = x;
        }
    }
}

// The persistent MC3 run's spurt bounds: the next spurt [next, end) into the
// run parameters (one thread, first node of the outer loop's body).
__global__ void mc3_begin_kernel(Mc3Dev* m, RunParams* rp) {
    const int64_t it0 = m->next;
    int64_t it1 = m->period > 0 ? (it0 / m->period + 1) * m->period : m->total;
    if (it1 > m->total) it1 = m->total;
    rp->first = it0;
    rp->end = it1;
}

// After the spurt and its exchange: the next spurt, and (set) whether the
// outer loop runs again.
__global__ void mc3_end_kernel(Mc3Dev* m, const RunParams* rp, cudaGraphConditionalHandle h, int set) {
    m->next = rp->end;
    if (set) cudaGraphSetConditional(h, m->next < m->total ? 1u : 0u);
}

cudaError_t launch_mc3_exchange(const ProblemDev& P, Mc3Dev* m, const RunParams* rp, int64_t it_end, int C,
                                uint32_t* dg, double* fag, double* rec, int64_t* accept, int64_t* propose,
                                cudaStream_t s) {
    mc3_pick_kernel<<<1, 1, 0, s>>>(m, rp, it_end, C);
    cudaError_t e = launch_loglik_parts(P, dg, nullptr, nullptr, 4, fag, rec, s, m);
    if (e != cudaSuccess) return e;
    mc3_decide_kernel<<<1, 256, 0, s>>>(m, P.M, P.marker_trans, fag, rec, dg, (size_t)P.M * P.W, accept, propose);
    return cudaGetLastError();
}

// Set conditional handles of the graph this kernel is a node of (up to 64 per launch).
struct CondSet {
    cudaGraphConditionalHandle h[64];
    int n;
    unsigned v;
};

__global__ void cond_set_kernel(CondSet cs) {
    if ((int)threadIdx.x < cs.n) cudaGraphSetConditional(cs.h[threadIdx.x], cs.v);
}

cudaError_t launch_cond_set(const cudaGraphConditionalHandle* h, int n, unsigned v, cudaStream_t s) {
    for (int i = 0; i < n; i += 64) {
        CondSet cs;
        cs.n = n - i < 64 ? n - i : 64;
        cs.v = v;
        for (int k = 0; k < cs.n; ++k) cs.h[k] = h[i + k];
        cond_set_kernel<<<1, 64, 0, s>>>(cs);
    }
    return cudaGetLastError();
}

cudaError_t launch_mc3_begin(Mc3Dev* m, RunParams* rp, cudaStream_t s) {
    mc3_begin_kernel<<<1, 1, 0, s>>>(m, rp);
    return cudaGetLastError();
}

cudaError_t launch_mc3_end(Mc3Dev* m, const RunParams* rp, cudaGraphConditionalHandle h, int set, cudaStream_t s) {
    mc3_end_kernel<<<1, 1, 0, s>>>(m, rp, h, set);
    return cudaGetLastError();
}

cudaError_t launch_swap_graphs(uint32_t* dg, size_t words, int a, int b, cudaStream_t s) {
    int64_t grid = (int64_t)((words + 255) / 256);
    if (grid > 1024) grid = 1024;
    swap_graphs_kernel<<<(int)grid, 256, 0, s>>>(dg, words, a, b);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Kernels of the run graph: every chain iterates on its own inside a WHILE
// node (MarkovChain::run, markov_chain.cc:335-392, per replicate chain).
// ---------------------------------------------------------------------------
__global__ void run_init_kernel(const RunParams* rp, int64_t* it, int C) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < C) it[c] = rp->first;
}

// Start of an iteration of chain c: the L/M choice (the same draw as
// choose_kernel), the meiosis order of an M-sweep (the same draws and swaps as
// shuffle_kernel, the uniforms generated by the warp), the chain's Philox key
// and whether the iteration scores.  One warp.
__global__ void chain_iter_kernel(const RunParams* rp, const int64_t* it_arr, int c, uint64_t* key,
                                  const int32_t* base, int nm, int32_t* order, const double* temp,
                                  cudaGraphConditionalHandle hsw, cudaGraphConditionalHandle hscore) {
    extern __shared__ double su[];
    const int lane = threadIdx.x;
    const int64_t it = it_arr[c];
    if (it >= rp->end) {
        if (lane == 0) {
            cudaGraphSetConditional(hsw, 2);   // neither sweep
            cudaGraphSetConditional(hscore, 0);
        }
        return;
    }
    const uint64_t seed = rp->seed, iter = (uint64_t)it;
    const uint64_t hic = ((uint64_t)c << 40) ^ (iter << 4) ^ 7u;
    const bool is_l = philox_u01(seed, hic, 0) < rp->lprob;
    if (!is_l) {
        const uint64_t hi = ((uint64_t)c << 40) ^ (iter << 4) ^ 3u;
        for (int i = 1 + lane; i < nm; i += 32) su[i] = philox_u01(seed, hi, (uint64_t)i);
        for (int i = lane; i < nm; i += 32) order[i] = base[i];
        __syncwarp();
        if (lane == 0)
            for (int i = nm - 1; i > 0; --i) {
                int j = (int)(su[i] * (double)(i + 1));
                if (j > i) j = i;
                const int32_t t = order[i];
                order[i] = order[j];
                order[j] = t;
            }
    }
    if (lane == 0) {
        key[0] = seed;
        key[1] = iter;
        cudaGraphSetConditional(hsw, is_l ? 0 : 1);
        // only the chains at temperature 1 are scored (markov_chain.cc:173-174)
        cudaGraphSetConditional(hscore, (it >= rp->burnin && it % rp->period == 0 && temp[c] == 1.0) ? 1 : 0);
    }
}

__global__ void chain_advance_kernel(const RunParams* rp, int64_t* it_arr, int c, cudaGraphConditionalHandle hwhile) {
    const int64_t next = it_arr[c] + 1;
    it_arr[c] = next;
    cudaGraphSetConditional(hwhile, next < rp->end ? 1 : 0);
}

// Fold the chains' LOD tables into the context's, chain by chain
// (LODscores::merge_results, lod_score.h:98-105), and clear them.
__global__ void chain_merge_kernel(double* acc_c, uint8_t* init_c, int C, int64_t npos, double* acc, uint8_t* init) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npos; p += (int64_t)gridDim.x * blockDim.x) {
        double a = acc[p];
        uint8_t ini = init[p];
        for (int c = 0; c < C; ++c) {
            const size_t q = (size_t)c * npos + p;
            if (!init_c[q]) continue;
            a = ini ? log_sum(a, acc_c[q]) : acc_c[q];
            ini = 1;
            init_c[q] = 0;
        }
        acc[p] = a;
        init[p] = ini;
    }
}

cudaError_t launch_run_init(const RunParams* rp, int64_t* it, int C, cudaStream_t s) {
    run_init_kernel<<<(C + 127) / 128, 128, 0, s>>>(rp, it, C);
    return cudaGetLastError();
}

cudaError_t launch_chain_iter(const RunParams* rp, const int64_t* it, int c, uint64_t* key, const int32_t* base,
                              int nm, int32_t* order, const double* temp, cudaGraphConditionalHandle hsw,
                              cudaGraphConditionalHandle hscore, cudaStream_t s) {
    chain_iter_kernel<<<1, 32, sizeof(double) * (nm > 0 ? nm : 1), s>>>(rp, it, c, key, base, nm, order, temp, hsw,
                                                                        hscore);
    return cudaGetLastError();
}

cudaError_t launch_chain_advance(const RunParams* rp, int64_t* it, int c, cudaGraphConditionalHandle hwhile,
                                 cudaStream_t s) {
    chain_advance_kernel<<<1, 1, 0, s>>>(rp, it, c, hwhile);
    return cudaGetLastError();
}

cudaError_t launch_chain_merge(double* acc_c, uint8_t* init_c, int C, int64_t npos, double* acc, uint8_t* init,
                               cudaStream_t s) {
    int64_t grid = (npos + 255) / 256;
    if (grid > 4096) grid = 4096;
    chain_merge_kernel<<<(int)grid, 256, 0, s>>>(acc_c, init_c, C, npos, acc, init);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
size_t lsampler_smem_per_warp(const ProblemDev& P) {
    return P.ls_fast ? ls_warp_bytes<float>(P) : ls_warp_bytes<double>(P);
}

size_t lsampler_smem_shared(const ProblemDev& P) { return ls_tables_bytes(P); }


template <typename T, int G>
static cudaError_t launch_lsampler_g(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* loci,
                                     int nloci, const Draws& d, const uint8_t* sel, int want, int* status,
                                     cudaStream_t s, int grid_cap, int wpb) {
    const int tpb = wpb * (32 / G);
    const size_t smem = ls_tables_bytes(P) + (size_t)tpb * ls_warp_bytes<T>(P);
    {
        cudaError_t e = ensure_smem((const void*)lsampler_kernel<T, G>, smem);
        if (e != cudaSuccess) return e;
    }
    const int64_t ntask = (int64_t)nchain * nloci;
    int64_t grid = (ntask + tpb - 1) / tpb;
    if (grid > grid_cap) grid = grid_cap;
    if (grid < 1) grid = 1;
    lsampler_kernel<T, G><<<(int)grid, wpb * 32, smem, s>>>(P, dg, first, nchain, loci, nloci, d, sel, want, status);
    return cudaGetLastError();
}

// The most L-sampler tasks an SM keeps resident, over the three lane groups,
// for blocks of wpb warps' worth of tasks (launch_lsampler's shapes): the
// occupancy of each kernel with its shared memory and registers.
template <typename T, int G>
static int ls_resident_g(const ProblemDev& P, int wpb) {
    const int tpb = wpb * (32 / G);
    const size_t smem = ls_tables_bytes(P) + (size_t)tpb * ls_warp_bytes<T>(P);
    if (ensure_smem((const void*)lsampler_kernel<T, G>, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, (const void*)lsampler_kernel<T, G>, wpb * 32, smem) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return blocks * tpb;
}

template <typename T>
static int ls_resident_t(const ProblemDev& P, int wpb) {
    const int a = ls_resident_g<T, 32>(P, wpb);
    const int b = ls_resident_g<T, 16>(P, wpb > 1 ? wpb / 2 : 1);
    const int c = ls_resident_g<T, 8>(P, wpb > 3 ? wpb / 4 : 1);
    return std::max(a, std::max(b, c));
}

int lsampler_resident_tasks(const ProblemDev& P, int wpb) {
    return P.ls_fast ? ls_resident_t<float>(P, wpb) : ls_resident_t<double>(P, wpb);
}

// lanes = 32, 16 or 8 lanes per (chain, locus) task; all draw the same graphs.
cudaError_t launch_lsampler(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* loci, int nloci,
                            const double* u, int64_t ucs, int64_t uls, uint64_t seed, uint64_t iter,
                            const uint8_t* sel, int want, int* status, cudaStream_t s, int grid_cap, int wpb,
                            const uint64_t* key, int lanes) {
    Draws d{u, ucs, uls, seed, iter, 1, key};
    if (lanes == 8) {
        // four tasks per warp: a quarter of the warps per block keeps the block's shared memory
        const int w8 = wpb > 3 ? wpb / 4 : 1;
        if (P.ls_fast) return launch_lsampler_g<float, 8>(P, dg, first, nchain, loci, nloci, d, sel, want, status, s,
                                                          grid_cap, w8);
        return launch_lsampler_g<double, 8>(P, dg, first, nchain, loci, nloci, d, sel, want, status, s, grid_cap, w8);
    }
    if (lanes == 16) {
        // two tasks per warp: half as many warps per block keeps the block's shared memory
        const int w16 = wpb > 1 ? wpb / 2 : 1;
        if (P.ls_fast) return launch_lsampler_g<float, 16>(P, dg, first, nchain, loci, nloci, d, sel, want, status, s,
                                                           grid_cap, w16);
        return launch_lsampler_g<double, 16>(P, dg, first, nchain, loci, nloci, d, sel, want, status, s, grid_cap, w16);
    }
    if (P.ls_fast)
        return launch_lsampler_g<float, 32>(P, dg, first, nchain, loci, nloci, d, sel, want, status, s, grid_cap, wpb);
    return launch_lsampler_g<double, 32>(P, dg, first, nchain, loci, nloci, d, sel, want, status, s, grid_cap, wpb);
}

// Keep each chain's best imputation: over the batch's passes in pass order,
// the first whose weight beats the best so far (SequentialImputation::run,
// sequential_imputation.cc:14-43: `tmp_prob > best_prob`, starting from
// LOG_ZERO); its graph is copied in.  One block per chain.
__global__ void si_select_kernel(const uint32_t* scratch, uint32_t* dg, int first, int nchain, size_t words,
                                 const double* w, double* best, int npass) {
    for (int cr = blockIdx.x; cr < nchain; cr += gridDim.x) {
        double bw = best[cr];
        int bq = -1;
        for (int q = 0; q < npass; ++q)
            if (w[(size_t)q * nchain + cr] > bw) {
                bw = w[(size_t)q * nchain + cr];
                bq = q;
            }
        __syncthreads();
        if (bq < 0) continue;
        const uint32_t* src = scratch + ((size_t)bq * nchain + cr) * words;
        for (size_t i = threadIdx.x; i < words; i += blockDim.x) dg[(size_t)(first + cr) * words + i] = src[i];
        __syncthreads();
        if (threadIdx.x == 0) best[cr] = bw;
    }
}

cudaError_t launch_si(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* starts,
                      const double* u, int64_t ucs, uint64_t seed, uint64_t pass, double* weights, int* status,
                      cudaStream_t s, int wpb, int npass, int64_t pass_stride, int grid_cap) {
    const size_t smem = ls_tables_bytes(P) + wpb * lsampler_smem_per_warp(P);
    {
        cudaError_t e = ensure_smem(P.ls_fast ? (const void*)si_kernel<float> : (const void*)si_kernel<double>, smem);
        if (e != cudaSuccess) return e;
    }
    Draws d{u, ucs, 0, seed, pass, 5, nullptr};
    int grid = (nchain * npass + wpb - 1) / wpb;
    if (grid > grid_cap) grid = grid_cap;
    if (P.ls_fast)
        si_kernel<float><<<grid, wpb * 32, smem, s>>>(P, dg, first, nchain, starts, d, 0, weights, status, npass,
                                                      pass_stride);
    else
        si_kernel<double><<<grid, wpb * 32, smem, s>>>(P, dg, first, nchain, starts, d, 0, weights, status, npass,
                                                       pass_stride);
    return cudaGetLastError();
}

cudaError_t launch_si_select(const uint32_t* scratch, uint32_t* dg, int first, int nchain, size_t words,
                             const double* w, double* best, int npass, cudaStream_t s) {
    si_select_kernel<<<nchain < 1024 ? nchain : 1024, 256, 0, s>>>(scratch, dg, first, nchain, words, w, best, npass);
    return cudaGetLastError();
}

template <typename IX, typename PP>
static cudaError_t launch_msampler_t(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* meioses,
                                     int64_t mstride, int nm, const double* u, int64_t ucs, uint64_t seed,
                                     uint64_t iter, const uint8_t* sel, int want, typename PP::T* raw, float* raw32,
                                     void* fb, uint8_t* badc, uint8_t* maps, int* status, int fag_threads, int exact,
                                     cudaStream_t s, const uint64_t* key, double* ubuf, int pairs) {
    const int fast = exact ? 0 : 1;
    Draws d{u, ucs, P.M, seed, iter, 2, key};
    cudaError_t e0 = cudaMemsetAsync(badc, 0, (size_t)nchain, s);
    if (e0 != cudaSuccess) return e0;
    const size_t smem = fag_block_bytes(P.N, P.F, fag_threads, fast);
    {
        cudaError_t e = ensure_smem((const void*)fag_kernel<IX, PP>, smem);
        if (e != cudaSuccess) return e;
    }
    const int scan_threads = ffbs_scan_threads(P.M);
    size_t scan_smem = ffbs_scan_smem(P.M);
    int staged = 1;
    if (scan_smem > 200 * 1024) {   // long maps: read the chain's arrays from global memory
        scan_smem = ffbs_scan_scratch(scan_threads);
        staged = 0;
    }
    if (!exact) {
        cudaError_t e = ensure_smem((const void*)ffbs_scan_kernel, scan_smem);
        if (e != cudaSuccess) return e;
    }
    const int64_t ntask = (int64_t)nchain * P.M;
    const int grid = (int)((ntask + fag_threads - 1) / fag_threads);
    // fast mode: one warp per (chain, locus), else the thread-per-locus kernel
    // in log2 (component counts are 13-bit fields)
    // two loci per warp (16 lanes each: 17% fewer instructions per locus, 30%
    // longer per launch) when the caller asks for throughput and a column
    // fits in 16 words (with longer columns read from global memory and the
    // block's shared memory doubled, the 400-member pedigree's M-sweeps were
    // 16% slower than with 32 lanes)
    const int G = pairs && P.W <= 16 ? 16 : 32;
    const int eb = fagw_label_bytes(P.F);
    const size_t wsm = fagw_block_bytes(P.N, P.F, G, eb);
    const bool warp_like = !exact && wsm <= 200 * 1024 && 2 * P.F < 8192;
    const void* fk = G == 16 ? (eb == 1 ? (const void*)fag_warp_kernel<16, uint8_t> : (const void*)fag_warp_kernel<16, uint16_t>)
                             : (eb == 1 ? (const void*)fag_warp_kernel<32, uint8_t> : (const void*)fag_warp_kernel<32, uint16_t>);
    if (warp_like) {
        cudaError_t e = ensure_smem(fk, wsm);
        if (e != cudaSuccess) return e;
    }
    const int lpb = kFagWarpsPerBlock * (32 / G);   // loci per block
    const dim3 wgrid((unsigned)((P.M + lpb - 1) / lpb), (unsigned)nchain);
    double* upre = warp_like ? ubuf : nullptr;
    for (int j = -1; j < nm; ++j) {
        if (!warp_like)
            fag_kernel<IX, PP><<<grid, fag_threads, smem, s>>>(P, dg, first, nchain, meioses, mstride, j, sel, want,
                                                               raw, exact ? nullptr : raw32, badc, status, fast);
        else {
            float* rawf = (float*)raw;
            void* args[] = {(void*)&P, (void*)&dg, (void*)&first, (void*)&meioses, (void*)&mstride, (void*)&j,
                            (void*)&d, (void*)&sel, (void*)&want, (void*)&rawf, (void*)&raw32, (void*)&badc,
                            (void*)&status, (void*)&upre};
            cudaError_t e = cudaLaunchKernel(fk, wgrid, dim3(kFagWarpsPerBlock * 32), args, wsm, s);
            if (e != cudaSuccess) return e;
        }
        if (j < 0) continue;
        if (exact)
            ffbs_kernel<double><<<nchain, 32, 0, s>>>(P, dg, first, nchain, meioses, mstride, j, d, sel, want, badc,
                                                      (const double*)raw, nullptr, (double*)fb);
        else
            ffbs_scan_kernel<<<nchain, scan_threads, scan_smem, s>>>(P, dg, first, nchain, meioses, mstride, j, d, sel,
                                                                     want, badc, raw32, (float*)fb, maps, staged,
                                                                     upre);
    }
    return cudaGetLastError();
}

// log2 of each chain's major and minor allele frequency at each locus, in
// the founder-allele kernel's arithmetic (FP32 logs of the rounded frequencies)
__global__ void lfreq_kernel(const double* minor, float2* out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double m = minor[i];
        out[i] = make_float2(log2f((float)(1.0 - m)), log2f((float)m));
    }
}

cudaError_t launch_lfreq(const double* minor, float2* out, int64_t n, cudaStream_t s) {
    int64_t grid = (n + 255) / 256;
    if (grid > 4096) grid = 4096;
    if (grid < 1) grid = 1;
    lfreq_kernel<<<(int)grid, 256, 0, s>>>(minor, out, n);
    return cudaGetLastError();
}

cudaError_t launch_set_key(uint64_t* key, uint64_t seed, uint64_t iter, cudaStream_t s) {
    set_key_kernel<<<1, 1, 0, s>>>(key, seed, iter);
    return cudaGetLastError();
}

cudaError_t launch_msampler(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* meioses,
                            int64_t mstride, int nm, const double* u, int64_t ucs, uint64_t seed, uint64_t iter,
                            const uint8_t* sel, int want, double* raw64, float* raw32, void* fb, uint8_t* badc,
                            uint8_t* maps, int* status, int fag_threads, int exact, cudaStream_t s,
                            const uint64_t* key, double* ubuf, int pairs) {
    // the fast mode keeps log2 likelihoods as floats in the first half of the raw buffer
    float* rawl = (float*)raw64;
    if (2 * P.F <= 255) {
        if (exact)
            return launch_msampler_t<uint8_t, ProbExact>(P, dg, first, nchain, meioses, mstride, nm, u, ucs, seed,
                                                         iter, sel, want, raw64, raw32, fb, badc, maps, status,
                                                         fag_threads, exact, s, key, ubuf, pairs);
        return launch_msampler_t<uint8_t, ProbLog2>(P, dg, first, nchain, meioses, mstride, nm, u, ucs, seed, iter,
                                                    sel, want, rawl, raw32, fb, badc, maps, status, fag_threads,
                                                    exact, s, key, ubuf, pairs);
    }
    if (exact)
        return launch_msampler_t<uint16_t, ProbExact>(P, dg, first, nchain, meioses, mstride, nm, u, ucs, seed, iter,
                                                      sel, want, raw64, raw32, fb, badc, maps, status, fag_threads,
                                                      exact, s, key, ubuf, pairs);
    return launch_msampler_t<uint16_t, ProbLog2>(P, dg, first, nchain, meioses, mstride, nm, u, ucs, seed, iter, sel,
                                                 want, rawl, raw32, fb, badc, maps, status, fag_threads, exact, s,
                                                 key, ubuf, pairs);
}

size_t fag_smem(int N, int F, int threads, int fast) { return fag_block_bytes(N, F, threads, fast); }

cudaError_t launch_lod(const ProblemDev& P, int precision, const uint32_t* graphs, int64_t graph_words, int G,
                       double* vals, int* status, cudaStream_t s, int grid_cap, int wpb) {
    const int64_t ntask = (int64_t)G * (P.M - 1) * P.n_lod;
    int64_t grid = (ntask + wpb - 1) / wpb;
    if (grid > grid_cap) grid = grid_cap;
    if (grid < 1) grid = 1;
    if (precision == 0) {
        const size_t smem = (size_t)wpb * P.arena * sizeof(double);
        {
            cudaError_t e = ensure_smem((const void*)lod_kernel<double, false>, smem);
            if (e != cudaSuccess) return e;
        }
        lod_kernel<double, false><<<(int)grid, wpb * 32, smem, s>>>(P, graphs, graph_words, G, vals, status);
    } else if (precision == 2) {   // FP64 with per-rfunction power-of-two rescaling
        const size_t smem = (size_t)wpb * P.arena * sizeof(double);
        {
            cudaError_t e = ensure_smem((const void*)lod_kernel<double, true>, smem);
            if (e != cudaSuccess) return e;
        }
        lod_kernel<double, true><<<(int)grid, wpb * 32, smem, s>>>(P, graphs, graph_words, G, vals, status);
    } else if (P.prog) {
        const int S = P.prog_threads;
        const size_t smem = (size_t)S * P.prog_slots * sizeof(float);
        {
            cudaError_t e = ensure_smem((const void*)lod_prog_kernel, smem);
            if (e != cudaSuccess) return e;
        }
        int64_t pgrid = (ntask + S - 1) / S;
        if (pgrid > grid_cap * 4) pgrid = grid_cap * 4;
        lod_prog_kernel<<<(int)pgrid, S, smem, s>>>(P, graphs, graph_words, G, vals, status);
    } else {
        const size_t smem = (size_t)wpb * P.arena * sizeof(float);
        {
            cudaError_t e = ensure_smem((const void*)lod_kernel<float, true>, smem);
            if (e != cudaSuccess) return e;
        }
        lod_kernel<float, true><<<(int)grid, wpb * 32, smem, s>>>(P, graphs, graph_words, G, vals, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_trait_adjoint(const ProblemDev& P, const AdjDev& D, const uint32_t* graphs, int64_t graph_words,
                                 int64_t task0, int64_t ntask, double* grad, int* status, cudaStream_t s, int sms) {
    const int wpb = (int)std::max<int64_t>(1, std::min<int64_t>(4, (200 * 1024) / std::max(1, D.warp_bytes)));
    const size_t smem = (size_t)wpb * D.warp_bytes;
    {
        cudaError_t e = ensure_smem((const void*)trait_adjoint_kernel, smem);
        if (e != cudaSuccess) return e;
    }
    int blocks = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, (const void*)trait_adjoint_kernel, wpb * 32, smem) !=
            cudaSuccess || blocks < 1)
        blocks = 1;
    int64_t grid = (ntask + wpb - 1) / wpb;
    grid = std::min<int64_t>(grid, (int64_t)sms * blocks);
    trait_adjoint_kernel<<<(int)std::max<int64_t>(1, grid), wpb * 32, smem, s>>>(P, D, graphs, graph_words, task0,
                                                                                 ntask, grad, status);
    return cudaGetLastError();
}

// Resident blocks of 128 threads per SM of the one-thread-per-task form.
int trait_adjoint_thr_blocks() {
    int blocks = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, (const void*)trait_adjoint_thr_kernel, 128, 0) !=
            cudaSuccess || blocks < 1) {
        cudaGetLastError();
        blocks = 1;
    }
    return blocks;
}

// One block of 128 threads per 128 threads of the arena (arena_threads, the
// resident threads of every SM); the threads stride over the tasks.
cudaError_t launch_trait_adjoint_thr(const ProblemDev& P, const AdjDev& D, const uint32_t* graphs, int64_t graph_words,
                                     int64_t task0, int64_t ntask, double* grad, int* status, float* arena, int* expo,
                                     int64_t arena_threads, cudaStream_t s) {
    const int64_t blocks = arena_threads / 128;
    if (blocks < 1) return cudaErrorInvalidValue;
    trait_adjoint_thr_kernel<<<(int)blocks, 128, 0, s>>>(P, D, graphs, graph_words, task0, ntask, grad, status, arena,
                                                         expo);
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
