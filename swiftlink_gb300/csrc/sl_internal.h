// Internal layouts shared by the host code (sl_host.cc) and the kernels
// (sl_kernels.cu).  Not part of the public C ABI.
#pragma once

#include <stdint.h>

namespace sl {

enum { UU = 0, AA = 1, AU = 2, UA = 3 };                              // trait.h:21-27
enum { G_UNTYPED = 0, G_HETERO = 1, G_HOMOZ_A = 2, G_HOMOZ_B = 3 };   // genotype.h:26-31
enum { CHILD = 1, PARENT = 2, PARTNER = 3, LAST = 4 };                // peeling.h:16-22

// Status codes written by kernels into the context's device status word.
enum { ST_OK = 0, ST_ZERO_LIK = 1, ST_ILLEGAL_DG = 2, ST_LOD_NONPOS = 3 };

// One peel operation as the kernels read it.  Every field is warp-uniform.
struct OpDev {
    int32_t type, peel, c, n_prev, n_child;
    int32_t cut_at;    // opdata offset: c person ids (reference key order)
    int32_t prev_at;   // opdata offset: per prev [op index, c', pos_0 .. pos_{c'-1}]
    int32_t child_at;  // opdata offset: per child [child id, child pos, other-parent pos, peel is mother]
    int32_t mpos, fpos;  // child peel: cutset positions of the mother and the father
    int32_t mat_off;     // offset of this op's dense 4^c matrix in a task's arena
    int32_t scale_to;    // FP32 trait peel: binary exponent this op's largest cell is scaled to (see LI_SCALE)
    int32_t prev_ops_at; // opdata offset: the op index of each previous rfunction, in prev_at's order
};

// Everything a kernel needs about one problem; passed by value.
struct ProblemDev {
    int32_t N, F, M, K, n_lod, Nnf, W;   // W = 32-bit words per descent-graph column
    int32_t arena;                       // sum over ops of 4^c
    int32_t ls_arena;                    // the L-sampler's compact rfunctions: the largest, over loci, sum over
                                         // ops of their cells in legal states (sl_kernels.cu, ls_locus)
    int32_t ls_cap;                      // the part of them a task keeps in shared memory (<= ls_arena)
    int32_t ls_spill_cells;              // ls_arena - ls_cap: cells per task slot in the global spill buffer
    int64_t ls_spill_slots;              // task slots the spill buffer holds per chain
    int32_t ls_spill_chains;             // chains it has slots for
    void* ls_spill;                      // [chains][slots][ls_spill_cells] of the L-sampler's type, or null
    int32_t max_child;                   // max children of an op (>= 1)
    int32_t fag_bytes;                   // shared bytes one FAG evaluation needs
    double marker_trans;                 // log(0.5) * 2 * Nnf (descent_graph.cc:22)
    const int16_t* mother;               // [N], -1 for founders
    const int16_t* father;
    const uint8_t* geno;                 // [M][N]: bits 0-1 genotype code, bits 4-7 legal mask
    const int32_t* typ_off;              // [M] where each locus's typed members start in typ_ent (multiples of 8)
    const uint16_t* typ_ent;             // member << 2 | genotype code, heterozygotes first, members in order;
                                         // each list padded to a multiple of 8 entries (16-byte copies)
    const uint16_t* typ_cnt;             // [M] typed members per locus
    const uint16_t* typ_nhet;            // [M] heterozygotes per locus
    const uint8_t* typed;                // [N]
    const double* prior;                 // [M][4 genotype codes][4 states]
    const double* theta;                 // [M-1]
    const double* partial;               // [M-1]
    const double* minor;                 // [M]
    const double* dprob;                 // [N][4]
    const uint8_t* dmask;                // [N] bit v set when dprob[v] != 0
    const OpDev* ops;                    // [K]
    const int32_t* opdata;
    int32_t opdata_n;                    // words of opdata
    int32_t ls_stage_ops;                // the L-sampler copies ops and opdata to each block's shared memory
    const int16_t* fag_order;            // [N] parents before children, founders first
    const int16_t* lvl_order;            // [N] persons by generation level (founders = level 0)
    const int32_t* lvl_off;              // [n_lvl + 1] start of each level in lvl_order
    int32_t n_lvl;
    const int32_t* prog;                 // compiled trait peel (LI_* words), or null
    const float* pconst;                 // its constants
    int32_t prog_slots;                  // FP32 slots one task of the program needs
    int32_t prog_threads;                // threads per block of the program kernel
    int32_t lod_zero_ok;                 // a zero trait likelihood is a zero term, not an error
    int32_t ls_fast;                     // L-sampler in FP32 with per-rfunction rescaling
    // FP32 / precomputed copies for the fast kernels
    const float* theta_f;                // [M-1]
    const float* partial_f;              // [M-1]
    const double* log_theta;             // [M-1] log(theta)
    const double* log_itheta;            // [M-1] log(1 - theta)
    const float* prior_f;                // [M][4][4]
    // each chain's map at its MC3 temperature t (GeneticMap::set_temperature,
    // genetic_map.cc:95-117): theta_t = t theta + (1 - t) / 2, maf_t likewise
    const double* c_theta;               // [C][M-1]
    const float* c_theta_f;              // [C][M-1]
    const double* c_minor;               // [C][M]
    const float2* c_lfreq;               // [C][M] log2 of the major and the minor allele frequency, as floats
    const double* c_log_theta;           // [C][M-1] log(theta_t)
    const double* c_log_itheta;          // [C][M-1] log(1 - theta_t)
    const double* temp;                  // [C] temperatures
};

// Instructions of a compiled trait-peel program (the batched LOD scorer).
//   LI_REC  child dst            A[dst + 2i + j] = 0.25 * recombination term of child (i, j)
//   LI_SUM  dst n src...         A[dst] = sum of A[src]
//   LI_CELL dst nterm, then per term: nf const_index slot x nf
//                                A[dst] = sum over terms of const * product of A[slot]
//   LI_SCALE first count target  multiply A[first .. first+count) by 2^-e, e = ilogb(their max) - target:
//                                the largest value becomes 2^target.  A consumer multiplying n_prev
//                                rfunctions gets each scaled to 2^(120/n_prev - 4), so the product of
//                                its inputs' largest cells stays below 2^120 while the cells its terms
//                                actually read, often far below their rfunction's maximum, keep clear of
//                                FP32 underflow (scaling every maximum to 1 underflowed on a 400-member
//                                pedigree); the last rfunction's target is 0
//   LI_END  slot                 the likelihood
enum { LI_REC = 1, LI_SUM = 2, LI_CELL = 3, LI_SCALE = 4, LI_END = 5 };

// The trait-peel adjoint's plan (trait_adjoint_kernel, one warp per task,
// dense rfunctions in the warp's shared memory): where each op's matrix lives
// and which matrices the first forward pass keeps.  With one segment every
// matrix has its own place (store).  With several, an op's matrix is kept
// (its own place in the first part of the arena) only when a later segment
// reads it; the others share the second part, segment after segment, and are
// recomputed before their segment's reverse pass (recompute).
struct AdjDev {
    const int32_t* aoff;     // [K] float offset of op k's matrix; its adjoint is at aoff + half
    const int32_t* seg;      // [nseg + 1] first op of each segment, then K
    const uint8_t* keep;     // [K] 1 when the first forward pass's matrix stays in place
    const float* dprob;      // [N][4] disease probabilities (person.cc:85-119), FP32
    const float4* dgrad;     // [N][4] their derivatives by (pen HOMO_U, pen HETERO, pen HOMO_A, frequency)
    // every op's (cell, term) items, cell-major (item = 4 cell + term): word 0 the peel node's state
    // (bits 0-1) and, for a parent peel, each child's transmission mask (4 bits per child from bit 2,
    // children 7 on in the words after the offsets, 8 per word); then the arena offsets of the item's
    // factors in the previous rfunctions, two 16-bit offsets per word.  The same for every task.
    const uint32_t* items;
    const int32_t* item_at;  // [K] first word of op k's items
    int32_t nseg;
    int32_t half;            // floats of the matrices (the adjoints take as many)
    int32_t warp_bytes;      // shared bytes of one warp: matrices, adjoints, exponents [K], child bits,
                             // recombination terms [12 max_child]
};

// Words per item of op k in AdjDev::items.
__host__ __device__ inline int adj_item_words(int n_prev, int n_child) {
    return 1 + (n_prev + 1) / 2 + (n_child > 7 ? (n_child - 7 + 7) / 8 : 0);
}

// Options of a device-driven run, read by the run graph's kernels.
struct RunParams {
    int64_t first, end, burnin, period;
    double lprob;
    uint64_t seed;
};

// MC3 exchanges on the device (Mc3::run, mc3.cc:117-158): the spurts of a run
// captured as one graph launch, and the exchange after each full spurt.
struct Mc3Dev {
    int64_t next, total, period;   // the next spurt's first iteration; the run's end; the exchange period
    int64_t it_end;                // the end of the spurt the exchange follows
    uint64_t seed;
    int32_t active;                // the spurt just run ends on a multiple of the period: exchange
    int32_t r;                     // the proposed pair (r, r + 1)
    int32_t gch[4], tch[4];        // (graph chain, map chain): xx, yy, xy, yx
};

// What code outside sl_host.cc may read of a context.
struct CtxView {
    ProblemDev P;
    void* stream;        // cudaStream_t
    int* d_status;
    int device;
    int lod_precision;
    int lod_grid, lod_wpb;
};

}  // namespace sl
