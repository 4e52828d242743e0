/* TEST INFRASTRUCTURE ONLY: plain-C restatement of the reference's CPU hot
 * path, used as the checker for the CUDA kernels and as the timed CPU port.
 * It is never linked into, or called by, the product library.
 *
 * Parity is pinned against the reference's own code compiled in this repo's
 * development container (oracle/_ref, see oracle/Makefile) through the tests
 * in tests/test_oracle_pin.py and the fixtures in tests/golden/.
 *
 * Descent graphs use the reference's internal layout: int32
 * [locus][person][2] with offset 2N*locus + 2*person + parent
 * (descent_graph.h:35-37).  Persons are in the reference's internal order
 * (founders first, pedigree.cc:154-162).
 */
#ifndef SL_ORACLE_H_
#define SL_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int N, F, M, K, n_lod;
    const int32_t* mother;   /* [N] -1 for founders */
    const int32_t* father;   /* [N] */
    const int32_t* sex;      /* [N] 0 unsexed, 1 male, 2 female */
    const uint8_t* geno;     /* [M][N] unphased genotype code (0 untyped) */
    const uint8_t* typed;    /* [N] person has any typed marker */
    const uint8_t* legal;    /* [M][N] bit v set when phased state v survives genotype elimination */
    const double* prior;     /* [M][N][4] SamplerRfunction trait cache (person.cc:224-299) */
    const double* dprob;     /* [N][4] disease prob per phased state (person.cc:85-119) */
    const double* theta;     /* [M-1] */
    const double* partial;   /* [M-1] partial theta (genetic_map.cc:57-61) */
    const double* minor;     /* [M] minor allele frequency */
    /* peel operations in sequence order (CSR) */
    const int32_t* op_type;  /* 1 child, 2 parent, 3 partner, 4 last (peeling.h:16-22) */
    const int32_t* op_peel;
    const int32_t* cut_off;  /* [K+1] */
    const int32_t* cut;
    const int32_t* prev_off; /* [K+1] */
    const int32_t* prev;
    const int32_t* ch_off;   /* [K+1] children of a parent peel, cutset order */
    const int32_t* ch;
} slo_problem;

/* One L-sampler step at `locus` (locus_sampler2.cc:128-159).  Draws are read
 * from u in the reference's consumption order: one per op from the last op to
 * the first, then one per homozygous-parent meiosis in person order, maternal
 * before paternal.  Returns 0, or -1 on zero likelihood, -2 on draw overrun. */
int slo_lstep(const slo_problem* p, int32_t* dg, int locus, const double* u, int n_u, int* n_used);
/* A full L-sweep: every even locus, then every odd locus; locus l's draws
 * start at u[l * u_stride] (u_stride >= K + 2N).  Returns 0 or the first
 * failing step's code. */
int slo_lsweep(const slo_problem* p, int32_t* dg, const double* u, int u_stride);
/* L-steps at the listed loci in list order (in place, one workspace); the
 * i-th listed locus reads its draws from u[i * u_stride]. */
int slo_lsteps(const slo_problem* p, int32_t* dg, const int32_t* loci, int n, const double* u, int u_stride);
int slo_si(const slo_problem* p, int32_t* dg, int start, const double* u, int n_u, int* n_used, double* weight);

/* One M-sweep: reset at meioses[0] then one step per listed meiosis
 * (markov_chain.cc:345-351, meiosis_sampler.cc:17-203).  Step j reads its
 * draws from u[j*M ...] in backward-sampling order (locus M-1 first), skipping
 * loci where one filtered probability is exactly zero.  Returns 0 or -1. */
int slo_msweep(const slo_problem* p, int32_t* dg, const int32_t* meioses, int n, const double* u,
               int32_t* n_used);

/* LOD scoring of n_dgs descent graphs (peeler.cc:65-103, lod_score.h:74-105):
 * raw[(M-1)*n_lod] log-sum accumulators, the scored count and log P(T). */
int slo_lod(const slo_problem* p, const int32_t* dgs, int n_dgs, double* raw, uint32_t* count,
            double* trait_prob);
int slo_lod_ex(const slo_problem* p, const int32_t* dgs, int n_dgs, double* raw, uint32_t* count,
               double* trait_prob, int zero_ok);

/* The same scoring restricted to intervals [l0, l1): raw holds (l1-l0)*n_lod
 * accumulators, interval l0 first.  rescale = 1 divides every rfunction by
 * a power of two after it is complete and carries the exponents (an FP64 peel
 * that does not underflow on pedigrees of hundreds of members, where the
 * reference's plain peel does and Peeler::process exits, peeler.cc:89-92);
 * rescale = 0 is the plain peel.  Returns 0, -1 on a zero likelihood (unless
 * zero_ok), -2 on a bad range. */
int slo_lod_range(const slo_problem* p, const int32_t* dgs, int n_dgs, int l0, int l1, int rescale, double* raw,
                  uint32_t* count, double* trait_prob, int zero_ok);

/* Founder-allele-graph likelihood of one descent-graph column
 * (founder_allele_graph4.cc:34-442); 0.0 when the column is illegal. */
double slo_fag_likelihood(const slo_problem* p, const int32_t* dg, int locus);

/* log-likelihood of a whole descent graph (descent_graph.cc:184-267) */
double slo_loglik(const slo_problem* p, const int32_t* dg);

/* The smallest |draw - decision boundary| met by the sampler calls since the
 * last reset (L-step genotype and indicator draws, M-step backward draws):
 * test instrumentation for checking samplers that round differently. */
void slo_margin_reset(void);
double slo_margin(void);
/* per_locus (M doubles, or NULL to stop): each M-step's backward pass writes
 * the margin of its draw at every locus (1 where it takes none) */
void slo_margin_log(double* per_locus);

/* Philox4x32-10 uniform in [0,1) for (key, counter) (Salmon et al., SC'11) */
double slo_philox_uniform(uint64_t key, uint64_t c_hi, uint64_t c_lo);

#ifdef __cplusplus
}
#endif

#endif
