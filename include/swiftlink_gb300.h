/*
 * swiftlink_gb300: GB300-native (sm_103a) kernels for the MCMC hot path of
 * SwiftLink multipoint linkage analysis -- the locus (L-) sampler, the meiosis
 * (M-) sampler and the trait-peeling LOD scorer -- behind a plain C ABI.
 *
 * Conventions
 *  - Every call returns SL_OK (0) or a negative SL_E* code; nothing aborts.
 *    sl_last_error() gives a one-line reason for the last failure on a context.
 *  - The caller owns every host array passed in; the context owns its device
 *    buffers.  A context is bound to one device and one CUDA stream and is not
 *    thread-safe (the reference calls its GPU wrapper from the OpenMP master
 *    thread only, markov_chain.cc:385-388).
 *  - Persons are in the reference's internal order: founders first
 *    (pedigree.cc:154-162).  Phased states use the reference's enum
 *    {UU=0, AA=1, AU=2, UA=3}, first letter = maternal-origin allele
 *    (trait.h:21-27); unphased genotypes are {UNTYPED=0, HETERO=1, HOMOZ_A=2,
 *    HOMOZ_B=3} (genotype.h:26-31).
 *  - Descent graphs cross the boundary in the reference's internal layout,
 *    int32 [locus][person][2] with offset 2N*locus + 2*person + parent
 *    (descent_graph.h:35-37, DescentGraph::get_internal_ptr), one graph after
 *    another for multi-graph calls.  On the device they are bit-packed.
 *  - Uniform draws for the bit-exact sampler entry points are supplied by the
 *    caller in the order the reference consumes get_random()
 *    (random.h:12-13): see each entry point.
 */
#ifndef SWIFTLINK_GB300_H_
#define SWIFTLINK_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SL_OK 0
#define SL_EINVAL -1      /* bad argument or unsupported problem */
#define SL_ECUDA -2       /* CUDA runtime failure */
#define SL_EZERO -3       /* zero likelihood (locus_sampler2.cc:137-142, peeler.cc:92-95) */
#define SL_EILLEGAL -4    /* illegal descent graph (meiosis_sampler.cc:33-36, 129-132) */
#define SL_ENOMEM -5      /* device allocation failed */
#define SL_ENODEV -6      /* no usable CUDA device */

/* Peel operation types, as in peeling.h:16-22 */
#define SL_CHILD_PEEL 1
#define SL_PARENT_PEEL 2
#define SL_PARTNER_PEEL 3
#define SL_LAST_PEEL 4

/* Sampler arithmetic */
#define SL_SAMPLER_EXACT 0     /* FP64 in the reference's operation order: bit-exact draws */
#define SL_SAMPLER_FAST 1      /* M-sampler filter in FP32 on normalised likelihood pairs */

/* LOD arithmetic */
#define SL_LOD_FP64 0          /* plain: FP64 trait peel, one warp per (graph, interval, offset) */
#define SL_LOD_FP32_RESCALED 1 /* batched: FP32 peel with per-rfunction power-of-two rescaling */
#define SL_LOD_FP64_RESCALED 2 /* FP64 peel with per-rfunction rescaling: the plain form for pedigrees whose
                                  unscaled likelihood underflows FP64 (no counterpart in the reference) */

typedef struct sl_ctx sl_ctx;

/*
 * One pedigree, its map and its peel sequence: the data the reference's
 * GPULodscores constructor mirrors to the device (gpu_lodscores.h:63-83,
 * gpu_lodscores.cc:106-527) plus what the samplers need.
 */
typedef struct sl_problem_desc {
    int32_t n_members;          /* N */
    int32_t n_founders;         /* F; persons 0..F-1 are the founders */
    int32_t n_markers;          /* M (>= 2) */
    int32_t lod_per_interval;   /* n, the -n option (defaults.h:22) */
    int32_t sex_linked;         /* must be 0: like the reference's -g path (main.cc:534-537) */
    const int32_t* mother;      /* [N] internal id of the mother, -1 for founders */
    const int32_t* father;      /* [N] */
    const int32_t* sex;         /* [N] 0 unsexed, 1 male, 2 female (types.h:22-26) */
    const uint8_t* typed;       /* [N] 1 if the person has any typed marker */
    const uint8_t* genotypes;   /* [M][N] unphased genotype codes */
    const uint8_t* legal;       /* [M][N] genotype-elimination masks, bit v = phased state v is
                                   possible (elimination.cc:41-395); NULL = computed here */
    const double* disease_prob; /* [N][4] Person::disease_prob (person.cc:85-119) */
    const double* theta;        /* [M-1] recombination fractions (genetic_map.cc:39-54) */
    const double* partial_theta;/* [M-1] (genetic_map.cc:57-61) */
    const double* minor_freq;   /* [M] minor-allele frequency per SNP */
    /* peel sequence in evaluation order (PeelSequenceGenerator::get_peel_order,
       peeling.h:25-339), compressed-row lists */
    int32_t n_ops;              /* K */
    const int32_t* op_type;     /* [K] SL_*_PEEL */
    const int32_t* op_peelnode; /* [K] */
    const int32_t* cutset_off;  /* [K+1] */
    const int32_t* cutset;      /* cutset members, reference key order */
    const int32_t* prev_off;    /* [K+1] */
    const int32_t* prev;        /* previous rfunctions feeding each op */
    const int32_t* children_off;/* [K+1] */
    const int32_t* children;    /* children of a parent peel, cutset order */
    /* disease model, needed only by the trait-peel adjoint (affection NULL = absent):
       Person::disease_prob follows from these (person.cc:85-119, disease_model.cc:139-187) */
    const int32_t* affection;   /* [N] 0 unknown, 1 unaffected, 2 affected (types.h:28-32) */
    double disease_freq;        /* disease-allele frequency */
    double penetrance[3];       /* penetrance of the HOMO_U, HETERO, HOMO_A traits (trait.h:13-17) */
} sl_problem_desc;

typedef struct sl_options {
    int32_t device;             /* CUDA device ordinal */
    int32_t n_chains;           /* descent graphs held on the device (replicates x temperatures) */
    int32_t lod_precision;      /* SL_LOD_FP64 or SL_LOD_FP32_RESCALED */
    int32_t sampler_precision;  /* SL_SAMPLER_EXACT or SL_SAMPLER_FAST */
    int32_t lod_kernel;         /* SL_LOD_KERNEL_*: the batched scorer's kernel (0 = timed choice) */
    int32_t lod_flags;          /* SL_LOD_ZERO_OK or 0 */
    int32_t ls_kernel;          /* SL_LS_KERNEL_*: the FP32 L-sampler's kernel */
} sl_options;

/* Kernels of the FP32 L-sampler (SL_SAMPLER_FAST).  GENERIC interprets the
 * peel operations.  SPECIALISED compiles, at sl_create, a kernel with the
 * pedigree's operations written in as constants (NVRTC for sm_103a: seconds to
 * tens of seconds for a 100-member pedigree; sl_create fails if it does not
 * build); it performs the same rounded operations in the same order, so both
 * draw bit-identical graphs, and it pays off on long runs.  BACKGROUND starts
 * the same compile on a host thread at sl_create and runs the generic kernel
 * until the compile ends; the context then switches to the specialised kernel
 * at its next sl_run, sl_batch_run or L-sampler call (runs are issued in short
 * spans meanwhile, so a long run switches while it runs), or keeps the generic
 * kernel if the compile failed.  The graphs are the same either way.
 * sl_destroy waits for a compile still running.  Identical sources compile
 * once per process (a cache of recent kernels shared by all contexts). */
#define SL_LS_KERNEL_GENERIC 0
#define SL_LS_KERNEL_SPECIALISED 1
#define SL_LS_KERNEL_BACKGROUND 2
/* AUTO compiles the specialised kernel at sl_create (falling back to the
 * generic one if it does not build) and, before the first L-sampler work,
 * times one half-sweep of every chain with each kernel on a copy of the
 * chains' graphs and keeps the faster: the generic kernel stores only the
 * rfunction cells allowed by genotype elimination and wins on pedigrees with
 * large cutsets (hundreds of members), the specialised one on smaller ones. */
#define SL_LS_KERNEL_AUTO 3
/* GENERIC times 32, 16 and 8 lanes per (chain, locus) task (one, two or four
 * tasks per warp) before the first L-sampler work and keeps the fastest,
 * sharing the choice between contexts of one pedigree size class; these
 * three force one (all forms draw the same graphs). */
#define SL_LS_KERNEL_GENERIC32 4
#define SL_LS_KERNEL_GENERIC16 5
#define SL_LS_KERNEL_GENERIC8 6

/* A LOD position whose trait likelihood is 0 (an affected and an unaffected
 * member IBD 2 under a fully penetrant model, for instance) stops the
 * reference (Peeler::process, peeler.cc:89-92: exit(1)).  By default the
 * library reports it as SL_EZERO from the next synchronising call, after
 * counting the position as a zero term of the log-sum.  With SL_LOD_ZERO_OK
 * the zero term is counted and no error is raised (the adjoint then writes
 * NaN for that position). */
#define SL_LOD_ZERO_OK 1

/* Kernels of the batched (FP32-rescaled) LOD scorer.  AUTO compiles the
 * problem-specialised forms at sl_create and, at the first scoring, times each
 * candidate on that batch and keeps the fastest (the reference autotunes its
 * launch shape in GPULodscores, gpu_lodscores.cc:529-596).  The others force
 * one kernel; a forced specialised form that cannot be built fails sl_create. */
#define SL_LOD_KERNEL_AUTO 0
#define SL_LOD_KERNEL_INTERP 1      /* slot-program interpreter */
#define SL_LOD_KERNEL_JIT_REG 2     /* specialised straight-line code, values in registers */
#define SL_LOD_KERNEL_JIT_SMEM 3    /* specialised straight-line code, values in shared memory */

/* Create a context; replaces GPULodscores::GPULodscores (gpu_lodscores.h:63-83). */
int sl_create(const sl_problem_desc* problem, const sl_options* options, sl_ctx** out);

/* Release every device buffer of the context (gpu_lodscores.h:95-99). */
void sl_destroy(sl_ctx* ctx);

/* One-line description of the last failure on ctx (thread-local when ctx is NULL). */
const char* sl_last_error(const sl_ctx* ctx);

/* Copy descent graphs of chains [first, first+n) in / out (int32 reference layout). */
int sl_set_descent_graphs(sl_ctx* ctx, int32_t first, int32_t n, const int32_t* dg);
int sl_get_descent_graphs(sl_ctx* ctx, int32_t first, int32_t n, int32_t* dg);

/* Per-locus, per-state priors the L-sampler uses (Person::get_trait_probability,
 * person.cc:224-299), [M][N][4]; lets callers check the host-side tables. */
int sl_get_trait_priors(sl_ctx* ctx, double* out);

/* Genotype-elimination masks used by the context, [M][N]. */
int sl_get_legal_masks(sl_ctx* ctx, uint8_t* out);

/*
 * L-sampler: Gibbs update of every meiosis indicator at one locus
 * (LocusSampler::set_locus_minimal + LocusSampler::step, locus_sampler2.cc:
 * 128-159; Sampler::step interface, sampler.h:62).
 *
 * sl_lsampler_loci updates, for each chain c in [first, first+n_chains) and each
 * listed locus, the descent graph in place.  The listed loci must be pairwise
 * non-adjacent (the reference's noninterferring rule, markov_chain.cc:406-416),
 * so they are independent and run concurrently.  Draws: for chain c and the
 * i-th listed locus, u[(c-first)*u_chain_stride + loci[i]*u_locus_stride ...],
 * consumed in the reference order: one per peel operation from the last to the
 * first (sampler_rfunction.cc:159-188), then one per meiosis whose parent has a
 * homozygous sampled state, in person order, maternal first
 * (locus_sampler2.cc:44-65, 93-125).  u_locus_stride >= K + 2N suffices.
 */
int sl_lsampler_loci(sl_ctx* ctx, int32_t first, int32_t n_chains, const int32_t* loci,
                     int32_t n_loci, const double* u, int64_t u_chain_stride,
                     int64_t u_locus_stride);

/* A full L-sweep: all even loci, then all odd loci (each a non-interfering
 * set), draws laid out as for sl_lsampler_loci. */
int sl_lsampler_sweep(sl_ctx* ctx, int32_t first, int32_t n_chains, const double* u,
                      int64_t u_chain_stride, int64_t u_locus_stride);

/*
 * M-sampler sweep (markov_chain.cc:345-351; MeiosisSampler::reset/step,
 * meiosis_sampler.cc:17-203): reset at meioses[0], then one Gibbs step per
 * listed meiosis (meiosis id = 2*(person-F) + parent).  Step j of chain c reads
 * draws from u[(c-first)*u_chain_stride + j*M ...] in backward order
 * (locus M-1 first), skipping loci where a filtered probability is exactly 0.
 */
int sl_msampler_sweep(sl_ctx* ctx, int32_t first, int32_t n_chains, const int32_t* meioses,
                      int32_t n_meioses, const double* u, int64_t u_chain_stride);

/*
 * LOD scoring (Peeler::process + LODscores::add, peeler.cc:79-103,
 * lod_score.h:74-105; the reference GPU path GPULodscores::calculate,
 * gpu_lodscores.cc:598-607).  Scores every interval and every one of the n
 * positions of the current descent graph of chains [first, first+n_chains),
 * accumulating log-likelihood ratios in FP64 log-sum form on the device.
 */
int sl_lod_score_chains(sl_ctx* ctx, int32_t first, int32_t n_chains);

/* Same, for n_graphs caller-supplied descent graphs (int32 reference layout),
 * scored in order. */
int sl_lod_score_graphs(sl_ctx* ctx, int32_t n_graphs, const int32_t* dgs);

/* Raw accumulators [(M-1)*n] in LODscores::get_raw form, the number of scored
 * graphs and log P(T) (GPULodscores::get_results, gpu_lodscores.cc:621-637). */
int sl_lod_results(sl_ctx* ctx, double* raw_logsum, uint64_t* count, double* trait_prob);

/* Clear the LOD accumulators and count. */
int sl_lod_reset(sl_ctx* ctx);

/*
 * Full MCMC run on the device (MarkovChain::run, markov_chain.cc:314-404) for
 * every chain, with uniform draws from a counter-based Philox4x32-10 stream
 * keyed by (seed, chain).  Each iteration picks an L-sweep with probability
 * lsampler_prob, else an M-sweep over the non-ignorable meioses in a shuffled
 * order; after burnin, every `period`-th iteration scores the chains whose
 * temperature is 1.
 */
typedef struct sl_run_options {
    int32_t iterations;
    int32_t burnin;
    int32_t scoring_period;
    int32_t first_iteration;    /* iteration index of the first step (for resumable runs) */
    double lsampler_prob;
    uint64_t seed;
    int32_t exchange_period;    /* MC3: iterations between exchanges of adjacent chains' graphs, 0 = none
                                   (Mc3::run, mc3.cc:83-162); an exchange follows every iteration count
                                   that is a multiple of it, so split runs exchange as one run does */
} sl_run_options;

/* MC3 temperatures, one per chain in exchange order (chain 0 the coldest; the
 * reference's default is t_i = 1 / (1 + 0.001 2^i) for i > 0, mc3.cc:38-46).
 * A chain at temperature t samples with theta_t = t theta + (1 - t) / 2 and
 * maf_t = t maf + (1 - t) / 2 (GeneticMap::set_temperature, genetic_map.cc:
 * 95-117); only chains at t = 1 are scored (markov_chain.cc:173-174). */
int sl_set_temperatures(sl_ctx* ctx, const double* temps);

/* Exchange statistics of adjacent pairs (c, c+1), c < n_chains - 1: proposals
 * and acceptances so far (mc3.cc:166-176). */
int sl_mc3_stats(sl_ctx* ctx, int64_t* accepted, int64_t* proposed);

/* log P(G, graph) of chain g's descent graph under chain t's map
 * (DescentGraph::get_likelihood2, descent_graph.h:78-84): the value the
 * exchange step compares.  LOG_ZERO (-DBL_MAX) for an illegal graph. */
int sl_chain_loglik(sl_ctx* ctx, int32_t graph_chain, int32_t map_chain, double* loglik);

int sl_run(sl_ctx* ctx, const sl_run_options* opt);

/* Wait for all work queued on the context's stream. */
int sl_synchronize(sl_ctx* ctx);

/* Device-side status word: 0 when every kernel finished cleanly. */
int sl_device_status(sl_ctx* ctx, int32_t* status);

/* Number of kernel launches the context has issued (for measurement). */
int64_t sl_launch_count(const sl_ctx* ctx);

/* The cudaStream_t the context enqueues all its work on. */
int sl_get_stream(sl_ctx* ctx, void** stream);

/* Per-kernel timing (the reference's *_MICROBENCHMARKING cudaEvent timers,
 * gpu_markov_chain.cc:1104-1140): while enabled, every launch is bracketed by
 * CUDA events on the context's stream; sl_profile_read returns the summed
 * device time and launch count of one kernel class and clears it. */
#define SL_KERNEL_LSAMPLER 0
#define SL_KERNEL_MSAMPLER 1
#define SL_KERNEL_LOD 2
#define SL_KERNEL_LOD_MERGE 3
#define SL_KERNEL_OTHER 4
int sl_profile(sl_ctx* ctx, int32_t enable);
int sl_profile_read(sl_ctx* ctx, int32_t kernel, double* total_ms, int64_t* launches);

/*
 * Host-side tables, no device needed (the checks a caller can run before
 * creating a context):
 *  - genotype-elimination masks [M][N] (GenotypeElimination::elimination,
 *    elimination.cc:41-183, 383-395);
 *  - per-locus L-sampler priors [M][N][4] (Person::populate_trait_prob_cache,
 *    person.cc:224-299, filled while parsing, pedigree_parser.cc:157);
 *  - log P(T), the trait peel without a descent graph (Peeler::calc_trait_prob,
 *    peeler.cc:65-73).
 */
int sl_problem_legal_masks(const sl_problem_desc* problem, uint8_t* out);
int sl_problem_trait_priors(const sl_problem_desc* problem, double* out);
int sl_problem_trait_prob(const sl_problem_desc* problem, double* out);

/* The batched LOD form's compiled trait-peel program (its construction is host
 * work), evaluated on the host in FP64 for one descent graph (int32 reference
 * layout), interval and position: the log-likelihood ratio the kernels add,
 * log r - recombination log-probability - marker transmission
 * (peeler.cc:79-103). */
int sl_problem_lod_program_eval(const sl_problem_desc* problem, const int32_t* dg, int32_t locus,
                                int32_t offset, double* out);

/*
 * LOD scoring that allocates nothing.  This entry point has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory at the
 * point where they score: hosts whose own allocator reserves the device's
 * memory up front and forbids further driver allocations, and latency-bound
 * loops where a cudaMalloc/cudaFree, which can synchronise the whole device,
 * would stall other streams.  It scores as sl_lod_score_graphs does, with the
 * kernel the context scores with (in the FP32-rescaled form, before the first
 * sl_lod_score_* call has timed the candidates, the specialised kernel with
 * values in registers if it was built, else the interpreter), but the
 * per-graph, per-position values live in a file-scope device array of
 * SL_NOALLOC_SCRATCH_BYTES (8 MiB) that every GPU loading the library holds
 * until exit, and the caller passes device buffers:
 *   d_graphs  n_graphs packed descent graphs, uint32 [n_graphs][M][W] with
 *             W = ceil(2 (N - F) / 32) and bit b = 2 (person - F) + parent of
 *             word b >> 5 in each locus column (padding bits zero);
 *   d_logsum  (M-1)*n doubles of LOD log-sum accumulators, set by the caller to
 *             -DBL_MAX before the first call (the empty LODscores state); each
 *             call adds the graphs' log-likelihood ratios in graph order.
 * n_graphs * (M-1) * n must not exceed SL_NOALLOC_SCRATCH_BYTES / 8; larger
 * requests return SL_EINVAL.  The work is queued on the context's stream;
 * sl_synchronize reports device errors.  The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) once for that device; the
 * calling thread's current device is the same after the call as before it.
 * All calls share the one array: calls that overlap on the GPU (several
 * contexts or streams at once) race on it.  The context's own accumulators
 * and count are not touched.
 */
#define SL_NOALLOC_SCRATCH_BYTES (8u << 20)
int sl_lod_score_device_graphs_noalloc(sl_ctx* ctx, int32_t n_graphs, const uint32_t* d_graphs,
                                       double* d_logsum);

/*
 * Adjoint of the trait peel (the reverse sum-product of TraitRfunction's
 * peel, trait_rfunction.cc:28-137; no counterpart kernel in the reference).
 * For each of n_graphs descent graphs (int32 reference layout) and each LOD
 * position (interval l, position o), grad[((g*(M-1) + l)*n + o)*6 + k] is the
 * derivative of log L, L the trait-peel likelihood at that position
 * (peeler.cc:79-91), with respect to
 *   k = 0, 1: theta_L and theta_R of the position (trait_rfunction.h:50-56);
 *   k = 2, 3, 4: the penetrances of HOMO_U, HETERO, HOMO_A;
 *   k = 5: the disease-allele frequency.
 * ptrait_grad[4] (may be NULL) receives d log P(T) / d (penetrances, frequency)
 * (Peeler::calc_trait_prob, peeler.cc:65-73).  Needs the disease-model fields
 * of the problem.  The peel is recomputed on the device in FP32 with
 * power-of-two rescaling, in one of three forms: one warp per (graph,
 * interval, position) with the rfunctions in shared memory; one thread per
 * position with them in a global arena (up to 4 GiB, a column per thread);
 * or the peel and its reverse written out for this pedigree and compiled
 * with NVRTC at the first call, in SL_ADJOINT_VARIANTS variants (one thread
 * per position, every rfunction in a global arena of up to 4 GiB; under the
 * default memory budget, or a budget whose plan keeps every rfunction, for
 * peels whose cutsets have at most 4 members).  The
 * first call with graphs times the forms on its first tasks and keeps the
 * fastest (sl_adjoint_info), unless sl_adjoint_set_form fixed one; the first
 * two follow the memory plan of sl_adjoint_memory (kept, or recomputed when
 * they do not fit).  The forms give the same values up to the order of FP32
 * additions.
 */
int sl_trait_backward(sl_ctx* ctx, int32_t n_graphs, const int32_t* dgs, double* grad, double* ptrait_grad);

/*
 * The adjoint's working memory.  Each task (graph, interval, position) keeps
 * the peel's rfunctions and their adjoints in its warp's shared memory.  When
 * every rfunction and its adjoint fit bytes_per_task (0: 32 KB), all are kept
 * from the forward pass (one segment); otherwise the peel operations are
 * split into segments, only rfunctions that a later segment reads are kept,
 * and each earlier segment's other rfunctions are recomputed from those
 * before its reverse pass -- forward cutsets recomputed instead of stored,
 * at the cost of one more forward pass.  The plan used: *segments (1 =
 * everything stored) and *used_bytes per task (either may be NULL).  Results
 * agree between plans within FP32 rounding.
 */
int sl_adjoint_memory(sl_ctx* ctx, int64_t bytes_per_task, int32_t* segments, int64_t* used_bytes);

/* The adjoint's form (SL_ADJOINT_WARP, SL_ADJOINT_THREAD or
 * SL_ADJOINT_SPECIALISED; 0 before the first call with graphs, and again
 * after sl_adjoint_memory or sl_adjoint_set_form) and the times of the timed
 * launch of each (milliseconds, 0 for a form not timed; any pointer may be
 * NULL). */
#define SL_ADJOINT_WARP 1
#define SL_ADJOINT_THREAD 2
#define SL_ADJOINT_SPECIALISED 3
int sl_adjoint_info(sl_ctx* ctx, int32_t* form, double* warp_ms, double* thread_ms, double* specialised_ms);

/* Fix the adjoint's form for the following calls (0: choose by timing, the
 * default), and for SL_ADJOINT_SPECIALISED its variant (0 to
 * SL_ADJOINT_VARIANTS - 1, see sl_problem_adjoint_source; ignored by the
 * other forms).  SL_ADJOINT_SPECIALISED needs cutsets of at most 4 members
 * and the default memory budget or a budget whose plan keeps every rfunction
 * (sl_adjoint_memory: one segment), else SL_EINVAL; a later budget whose plan
 * splits the peel returns the choice to timing.  If its NVRTC compile
 * fails, the next sl_trait_backward returns SL_EINVAL with the compiler's
 * log. */
int sl_adjoint_set_form(sl_ctx* ctx, int32_t form, int32_t variant);

/* The specialised adjoint: the operation shapes it was generated with (one
 * forward and one reverse function each), the variant in use (the fastest
 * when timed, the first when fixed; see sl_problem_adjoint_source; -1 before
 * it was built) and its registers per thread, and the compile time of its
 * variants in milliseconds (0 before it was needed, -1 if its compile
 * failed); any pointer may be NULL. */
int sl_adjoint_kernel_info(sl_ctx* ctx, int32_t* shapes, int32_t* variant, int32_t* regs, double* compile_ms);

/* The batched LOD scorer specialised to a problem (the kernel sl_create
 * compiles for an SL_LOD_FP32_RESCALED context), as CUDA C++ source (no
 * device needed): values in registers (shared = 0) or in a per-thread
 * shared-memory arena (shared = 1), `threads` per block (a multiple of 32),
 * lod_flags as sl_options' (SL_LOD_ZERO_OK).  Up to cap - 1 bytes and a
 * terminating zero into buf (buf may be NULL with cap 0), its length into
 * *len and the program's float slots into *slots; with compile != 0 it is
 * also compiled with NVRTC for sm_103a (milliseconds into *compile_ms;
 * SL_EINVAL with the compiler's log when it fails).  Any output pointer may
 * be NULL. */
int sl_problem_lod_source(const sl_problem_desc* problem, int32_t shared, int32_t threads, int32_t lod_flags,
                          int32_t compile, char* buf, int64_t cap, int64_t* len, int32_t* slots, double* compile_ms);

/* The specialised adjoint's CUDA C++ source for a problem (no device
 * needed), one of its SL_ADJOINT_VARIANTS variants (0: compiled for 4 blocks
 * of 128 threads per SM, 1: for 8): up to cap - 1 bytes and a terminating
 * zero into buf (buf may be NULL with cap 0), its length into *len and its
 * operation shapes into *shapes; with compile != 0 it is also compiled with
 * NVRTC for sm_103a (milliseconds into *compile_ms; SL_EINVAL with the
 * compiler's log when it fails).  Any output pointer may be NULL. */
#define SL_ADJOINT_VARIANTS 2
int sl_problem_adjoint_source(const sl_problem_desc* problem, int32_t variant, int32_t compile, char* buf,
                              int64_t cap, int64_t* len, int32_t* shapes, double* compile_ms);

/* The same adjoint for one graph and position evaluated on the host in FP64
 * (the reference gradient the device result is checked against); dg NULL
 * gives the gradient of log P(T) in grad[2..5]. */
int sl_problem_trait_backward_eval(const sl_problem_desc* problem, const int32_t* dg, int32_t locus,
                                   int32_t offset, double* grad);

/* The batched LOD kernel in use (SL_LOD_KERNEL_*; AUTO until the first
 * scoring has timed the candidates) and the milliseconds spent compiling the
 * specialised forms at sl_create. */
int sl_lod_kernel_info(sl_ctx* ctx, int32_t* kernel, double* compile_ms);

/* The L-sampler kernel in use (SL_LS_KERNEL_GENERIC or SL_LS_KERNEL_SPECIALISED)
 * and the milliseconds the specialised form took to compile (0 if none was
 * asked for; -1 while a background compile is still running; a background
 * compile that failed leaves GENERIC with its time, and its reason in
 * sl_last_error).  A background compile that has ended is taken up here. */
int sl_ls_kernel_info(sl_ctx* ctx, int32_t* kernel, double* compile_ms);

/* The L-sampler autotuner's outcome: the lanes per (chain, locus) task of the
 * generic kernel in use (32, 16 or 8; 0 when the specialised kernel runs) and
 * the timed half-sweep of each candidate in milliseconds, times_ms[0..3] =
 * 32, 16 and 8 lanes and the specialised kernel (0 for a candidate not timed,
 * and for all of them before the first L-sampler work or when a pedigree of
 * the same size class on this device was timed first).  Either pointer may
 * be NULL. */
int sl_ls_tuning(sl_ctx* ctx, int32_t* lanes, double* times_ms);

/*
 * A peel sequence for a pedigree (members founders first, mother/father -1 for
 * founders), in the form sl_problem_desc takes (replaces PeelSequenceGenerator::
 * build_peel_sequence, peel_sequence_generator.cc:273-310, and its op
 * construction, :57-250).  The order is a greedy minimum-cutset elimination
 * refined by exchanges of neighbours (the reference's is a randomised downhill
 * search); the operations' types, cutsets, previous functions and children
 * follow the reference's rules.  op_type/op_peelnode hold n entries, the
 * offsets n + 1, and cutset/prev/children at most `capacity` each (SL_ENOMEM
 * when that is too small).  Host only; needs no device.
 */
int sl_peel_sequence(int32_t n, const int32_t* mother, const int32_t* father, int32_t capacity, int32_t* op_type,
                     int32_t* op_peelnode, int32_t* cutset_off, int32_t* cutset, int32_t* prev_off, int32_t* prev,
                     int32_t* children_off, int32_t* children);

/*
 * Batches: contexts of different pedigrees (uneven sizes, each with its own
 * chains and temperatures) run together, one graph launch per spurt holding
 * every context's per-chain WHILE nodes (no reference counterpart: the
 * reference runs pedigrees one after another, linkage_program.cc:96-108).
 * sl_batch_run takes one set of run options for all; with exchange_period > 0
 * each context then makes its own MC3 exchange.  Results are read per context
 * (sl_lod_results, sl_get_descent_graphs), ordered after the batch.  The
 * contexts must outlive the batch and run without profiling.
 */
typedef struct sl_batch sl_batch;
int sl_batch_create(sl_ctx* const* ctxs, int32_t n, sl_batch** out);
int sl_batch_run(sl_batch* batch, const sl_run_options* opt);
void sl_batch_destroy(sl_batch* batch);

/*
 * Sequential imputation (SequentialImputation::run / LocusSampler::start_from,
 * sequential_imputation.cc:14-43, locus_sampler2.cc:214-241): legal starting
 * graphs.  sl_sequential_imputation runs one pass per listed chain from the
 * given start locus with the given draws (chain c's at draws + c *
 * chain_stride, consumed in order as get_random() would return them) and
 * writes each pass's weight (the sum of log peel results; -DBL_MAX if a locus
 * has likelihood 0).  sl_sequential_imputation_run runs `iterations` passes
 * per chain from the Philox stream and keeps each chain's best graph;
 * best_weights (may be NULL) receives the best weights.
 */
int sl_sequential_imputation(sl_ctx* ctx, int32_t first, int32_t n_chains, const int32_t* start_loci,
                             const double* draws, int64_t chain_stride, double* weights);
int sl_sequential_imputation_run(sl_ctx* ctx, int32_t iterations, uint64_t seed, double* best_weights);

/* Library version string. */
const char* sl_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SWIFTLINK_GB300_H_ */
