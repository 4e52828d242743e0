// Host side of the swiftlink_gb300 C ABI: validates a problem, builds the
// device tables (per-locus priors, genotype-elimination masks, peel-operation
// descriptors with gather maps), bit-packs descent graphs, and enqueues the
// kernels of sl_kernels.cu on the context's stream.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <cfloat>
#include <chrono>
#include <thread>
#include <type_traits>
#include <tuple>
#include <mutex>
#include <vector>

#include "../../include/swiftlink_gb300.h"
#include "sl_adjjit.h"
#include "sl_internal.h"
#include "sl_jit.h"
#include "sl_lsjit.h"

namespace sl {
// kernels (sl_kernels.cu)
size_t lsampler_smem_per_warp(const ProblemDev& P);
size_t lsampler_smem_shared(const ProblemDev& P);
int lsampler_resident_tasks(const ProblemDev& P, int wpb);
cudaError_t launch_lsampler(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* loci,
                            int nloci, const double* u, int64_t ucs, int64_t uls, uint64_t seed, uint64_t iter,
                            const uint8_t* sel, int want, int* status, cudaStream_t s, int grid_cap, int wpb,
                            const uint64_t* key = nullptr, int lanes = 32);
cudaError_t launch_msampler(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* meioses,
                            int64_t mstride, int nm, const double* u, int64_t ucs, uint64_t seed, uint64_t iter,
                            const uint8_t* sel, int want, double* raw64, float* raw32, void* fb, uint8_t* badc,
                            uint8_t* maps, int* status, int fag_threads, int exact, cudaStream_t s,
                            const uint64_t* key = nullptr, double* ubuf = nullptr, int pairs = 0);
cudaError_t launch_set_key(uint64_t* key, uint64_t seed, uint64_t iter, cudaStream_t s);
cudaError_t launch_lfreq(const double* minor, float2* out, int64_t n, cudaStream_t s);
cudaError_t launch_si(const ProblemDev& P, uint32_t* dg, int first, int nchain, const int32_t* starts,
                      const double* u, int64_t ucs, uint64_t seed, uint64_t pass, double* weights, int* status,
                      cudaStream_t s, int wpb, int npass, int64_t pass_stride, int grid_cap);
cudaError_t launch_si_select(const uint32_t* scratch, uint32_t* dg, int first, int nchain, size_t words,
                             const double* w, double* best, int npass, cudaStream_t s);
cudaError_t launch_run_init(const RunParams* rp, int64_t* it, int C, cudaStream_t s);
cudaError_t launch_chain_iter(const RunParams* rp, const int64_t* it, int c, uint64_t* key, const int32_t* base,
                              int nm, int32_t* order, const double* temp, cudaGraphConditionalHandle hsw,
                              cudaGraphConditionalHandle hscore, cudaStream_t s);
cudaError_t launch_loglik_parts(const ProblemDev& P, const uint32_t* dg, const int* gch, const int* tch, int npair,
                                double* fag_out, double* rec_out, cudaStream_t s, const Mc3Dev* m = nullptr);
cudaError_t launch_mc3_exchange(const ProblemDev& P, Mc3Dev* m, const RunParams* rp, int64_t it_end, int C,
                                uint32_t* dg, double* fag, double* rec, int64_t* accept, int64_t* propose,
                                cudaStream_t s);
cudaError_t launch_mc3_begin(Mc3Dev* m, RunParams* rp, cudaStream_t s);
cudaError_t launch_mc3_end(Mc3Dev* m, const RunParams* rp, cudaGraphConditionalHandle h, int set, cudaStream_t s);
cudaError_t launch_cond_set(const cudaGraphConditionalHandle* h, int n, unsigned v, cudaStream_t s);
cudaError_t launch_swap_graphs(uint32_t* dg, size_t words, int a, int b, cudaStream_t s);
cudaError_t launch_chain_advance(const RunParams* rp, int64_t* it, int c, cudaGraphConditionalHandle hwhile,
                                 cudaStream_t s);
cudaError_t launch_chain_merge(double* acc_c, uint8_t* init_c, int C, int64_t npos, double* acc, uint8_t* init,
                               cudaStream_t s);
size_t fag_smem(int N, int F, int threads, int fast);
cudaError_t launch_lod(const ProblemDev& P, int precision, const uint32_t* graphs, int64_t graph_words, int G,
                       double* vals, int* status, cudaStream_t s, int grid_cap, int wpb);
cudaError_t launch_lod_merge(const double* vals, int G, int64_t npos, double* acc, uint8_t* init, cudaStream_t s);
cudaError_t launch_trait_adjoint(const ProblemDev& P, const AdjDev& D, const uint32_t* graphs, int64_t graph_words,
                                 int64_t task0, int64_t ntask, double* grad, int* status, cudaStream_t s, int sms);
int trait_adjoint_thr_blocks();
cudaError_t launch_trait_adjoint_thr(const ProblemDev& P, const AdjDev& D, const uint32_t* graphs, int64_t graph_words,
                                     int64_t task0, int64_t ntask, double* grad, int* status, float* arena, int* expo,
                                     int64_t arena_threads, cudaStream_t s);
cudaError_t launch_shuffle(const int32_t* base, int nm, int32_t* out, int first, int nchain, uint64_t seed,
                           uint64_t iter, cudaStream_t s);
cudaError_t launch_choose(int first, int nchain, uint64_t seed, uint64_t iter, double lprob, uint8_t* is_l,
                          cudaStream_t s);
}  // namespace sl

using namespace sl;

namespace {
thread_local std::string g_err;
const size_t kSmemBudget = 200 * 1024;  // dynamic shared memory a block may use
}  // namespace

enum { LS_GEN32 = 0, LS_GEN16 = 1, LS_JIT = 2, LS_GEN8 = 3 };
static int ls_lanes(int choice) { return choice == LS_GEN16 ? 16 : (choice == LS_GEN8 ? 8 : 32); }

struct sl_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t lstream = nullptr;   // L-sweeps of device-driven runs, concurrent with M-sweeps
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int n_chains = 0;
    int lod_precision = 0;
    int sampler_precision = 0;
    int sms = 0;
    ProblemDev P{};
    // host copies
    std::vector<double> prior_table;     // [M][4][4]
    std::vector<double> theta_h, minor_h;   // the map at temperature 1
    std::vector<double> temps;           // [C] MC3 temperatures
    // MC3 exchange statistics per adjacent pair (mc3.cc:138-157), counted on the device
    std::vector<int64_t> swap_accept, swap_propose;   // host copies read by sl_mc3_stats
    int64_t* d_swap_acc = nullptr;    // [C-1]
    int64_t* d_swap_prop = nullptr;   // [C-1]
    Mc3Dev* d_mc3 = nullptr;          // the exchange's state: spurt bounds, proposal, pairs
    double* d_llfag = nullptr;        // [4][M] founder-allele-graph likelihoods of the exchange step
    double* d_llrec = nullptr;        // [4][M-1] recombination log-probabilities
    // an MC3 run as one launch: an outer WHILE node over spurts, each the run
    // nodes followed by the exchange
    cudaGraphExec_t mc3_graph = nullptr;
    int run_graph_epoch = 0, mc3_graph_epoch = 0;   // ls_epoch when each graph was captured
    std::vector<uint8_t> legal;          // [M][N]
    std::vector<int32_t> meioses;        // non-ignorable meioses (markov_chain.cc:70-80)
    std::vector<int32_t> even, odd;
    double trait_prob = 0.0;
    uint64_t lod_count = 0;
    int64_t launches = 0;
    // launch shapes
    int ls_wpb = 1, ls_grid = 1, lod_wpb = 1, lod_grid = 1, ms_threads = 32;
    // device buffers
    std::vector<void*> owned;
    uint32_t* d_dg = nullptr;
    double* d_acc = nullptr;
    uint8_t* d_init = nullptr;
    double* d_vals = nullptr;
    int vals_graphs = 0;
    uint32_t* d_graphs = nullptr;
    int graphs_cap = 0;
    double* d_u = nullptr;
    size_t u_cap = 0;
    int32_t* d_loci = nullptr;
    int32_t* d_even = nullptr;
    int32_t* d_odd = nullptr;
    int32_t* d_meioses = nullptr;
    int32_t* d_morder = nullptr;     // [C][nm] per-chain orders for device-driven sweeps
    int32_t* d_mlist = nullptr;      // staging for caller meiosis lists
    size_t mlist_cap = 0;
    double* d_raw = nullptr;
    float* d_raw32 = nullptr;
    double* d_fb = nullptr;
    uint8_t* d_badc = nullptr;
    uint8_t* d_maps = nullptr;       // [C][M] backward decision maps of the fast filter
    double* d_mu = nullptr;          // [C][M] the fast M-step's draws by index
    int* d_status = nullptr;
    uint8_t* d_sel = nullptr;
    uint32_t* h_stage = nullptr;     // pinned staging for packed descent graphs
    size_t h_stage_words = 0;
    // the M-sweep of device-driven runs as a graph: one branch per chain, so a
    // chain's filter overlaps other chains' founder-allele graphs
    cudaGraphExec_t ms_graph = nullptr;
    int64_t ms_graph_kernels = 0;
    uint64_t* d_key = nullptr;        // [2] seed and iteration read by the graph's kernels
    std::vector<cudaStream_t> cap_streams;
    std::vector<cudaEvent_t> cap_events;
    // the whole device-driven run as one graph: a WHILE node per chain
    cudaGraphExec_t run_graph = nullptr;
    RunParams* d_run = nullptr;
    int64_t* d_chain_it = nullptr;    // [C] each chain's next iteration
    uint64_t* d_keys = nullptr;       // [C][2] each chain's Philox seed and iteration
    double* d_acc_c = nullptr;        // [C][npos] each chain's LOD log-sums of the run
    uint8_t* d_init_c = nullptr;      // [C][npos]
    bool chain_tables_pending = false; // chain tables hold scores not yet merged into d_acc
    // trait-peel adjoint (present when the problem carries the disease model)
    bool has_adjoint = false;
    AdjDev adj{};
    std::vector<OpDev> adj_ops;       // host copies the plan is built from
    std::vector<int32_t> adj_od;      // their opdata
    std::vector<int32_t> adj_prev;    // [K+1] CSR offsets and the previous ops, for the plan's consumers
    std::vector<int32_t> adj_prevs;
    size_t adj_budget = 0;            // shared bytes per warp the plan must fit (0: the default)
    double* d_adjG = nullptr;        // [chunk][6] gradients
    int64_t adj_chunk = 0;
    // the adjoint's forms: one warp per task with its matrices in shared memory, one thread per
    // task with them in a global arena (a column per thread), or the peel's adjoint compiled for
    // this pedigree (one thread per task, sl_adjjit.cc; only under a plan that keeps every
    // matrix); chosen by timing the first call unless the caller fixed one (sl_adjoint_set_form)
    int adj_form = 0;                 // 0 not yet timed, SL_ADJOINT_WARP, _THREAD, _SPECIALISED
    int adj_form_req = 0;             // 0: by timing
    double adj_form_ms[3] = {0.0, 0.0, 0.0};
    float* d_adjA = nullptr;          // [2 half][threads] matrices and adjoints of the thread form
    int* d_adjE = nullptr;            // [K][threads] their exponents
    int64_t adj_thr = 0;              // threads the arena holds
    size_t adj_thr_bytes = 0;
    AdjJit adj_jit_v[kAdjJitVariants];   // the specialised form at each register budget
    int adj_jit_sel = 0;              // the variant in use (timed with the forms)
    int adj_jit_req = 0;              // the variant a fixed SL_ADJOINT_SPECIALISED form runs
    int adj_jit_state = 0;            // 0 not tried, 1 built, -1 its compile failed
    std::string adj_jit_log;
    float* d_adjJ = nullptr;          // its arena: blocks x adj_jit_block_floats
    int64_t adj_jit_blocks = 0;
    // batched LOD kernel: the interpreter, or a problem-specialised form
    int lod_kernel_req = SL_LOD_KERNEL_AUTO;
    JitLs jit_ls;                     // the FP32 L-sampler specialised to the pedigree (kern null: generic)
    double jit_ls_ms = 0.0;
    // SL_LS_KERNEL_BACKGROUND: the compile runs on ls_thread; the context takes it up (ls_adopt) at its
    // next run or L-sampler call after ls_pending turns 2
    std::thread ls_thread;
    std::atomic<int> ls_pending{0};             // 0 none, 1 compiling, 2 ended and not yet taken up
    std::shared_ptr<const JitBinary> ls_bin;    // written by ls_thread before ls_pending = 2
    double ls_thread_ms = 0.0;                  // likewise
    size_t ls_warp_bytes = 0;
    int jit_ls_wpb = 1;                  // warps per block of the specialised L-sampler (its own arena layout)
    int ls_epoch = 0;                           // kernel switches (graphs captured before are redone)
    // the L-sampler's kernel and lanes per task: the generic kernel with 32 or
    // 16 lanes, or the specialised one; chosen by timing (ls_tune) unless forced
    bool ls_tune_pending = false;
    int ls_choice = 0;                          // LS_GEN32, LS_GEN16, LS_GEN8, LS_JIT
    double ls_tune_ms[4] = {0.0, 0.0, 0.0, 0.0};   // one timed half-sweep with each (0: not timed)
    int lod_kernel_sel = SL_LOD_KERNEL_INTERP;   // AUTO while the first scoring has not timed them
    JitLod jit_reg, jit_smem;
    double jit_ms = 0.0;
    std::string err;
    // per-kernel event timing
    bool profiling = false;
    struct Mark { int kernel; cudaEvent_t a, b; };
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> event_pool;
    double prof_ms[5] = {0, 0, 0, 0, 0};
    int64_t prof_n[5] = {0, 0, 0, 0, 0};
};

namespace {
cudaEvent_t take_event(sl_ctx* c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
// Bracket one launch with events when profiling is on.
// Kernels one M-sweep of nm meioses launches for a chain: a reset, then per
// meiosis a likelihood and a filter kernel.
static int64_t msweep_kernels(const sl_ctx*, int nm) { return 1 + 2 * (int64_t)nm; }

// The fast M-step's likelihood kernel puts two loci in a warp (fewer
// instructions per locus, a longer launch) when the context holds enough
// chains for the GPU to be throughput-bound.
static int msampler_pairs(const sl_ctx* ctx) { return ctx->n_chains >= 8 ? 1 : 0; }

// An L-sampler launch: the kernel specialised to the pedigree when it was
// built, else the generic one.
static cudaError_t ls_launch(sl_ctx* ctx, int first, int nchain, const int32_t* loci, int nloci, const double* u,
                             int64_t ucs, int64_t uls, uint64_t seed, uint64_t iter, const uint8_t* sel, int want,
                             cudaStream_t s, const uint64_t* key = nullptr) {
    const ProblemDev& P = ctx->P;
    if (ctx->jit_ls.kern && ctx->ls_choice == LS_JIT)
        return jit_ls_launch(ctx->jit_ls, ctx->d_dg, first, nchain, loci, nloci, u, ucs, uls, seed, iter, key, sel,
                             want, ctx->d_status, P.geno, P.prior_f, P.c_theta_f, ctx->sms, s);
    return launch_lsampler(P, ctx->d_dg, first, nchain, loci, nloci, u, ucs, uls, seed, iter, sel, want, ctx->d_status,
                           s, ctx->ls_grid, ctx->ls_wpb, key, ls_lanes(ctx->ls_choice));
}

// Takes up a background compile of the specialised L-sampler that has ended:
// loads it into the context's device and drops the run graph captured with the
// generic kernel.  A compile or load that failed leaves the generic kernel and
// its reason in the context's last error.
static void ls_adopt(sl_ctx* ctx) {
    if (ctx->ls_pending.load(std::memory_order_acquire) != 2) return;
    ctx->ls_thread.join();
    ctx->ls_pending.store(0, std::memory_order_relaxed);
    ctx->jit_ls_ms = ctx->ls_thread_ms;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(ctx->device);
    std::string log;
    JitLs j;
    if (jit_ls_load(*ctx->ls_bin, ctx->jit_ls_wpb, ctx->ls_warp_bytes, &j, &log)) {
        ctx->err = "specialised L-sampler failed (the generic kernel runs): " + log.substr(0, 300);
    } else {
        ctx->jit_ls = j;
        ctx->ls_choice = LS_JIT;
        ctx->jit_ls.compile_ms = ctx->ls_thread_ms;
        ++ctx->ls_epoch;   // the run graphs are captured again at their next launch
    }
    ctx->ls_bin.reset();
    cudaSetDevice(cur);
}

static bool ls_compiling(const sl_ctx* ctx) { return ctx->ls_pending.load(std::memory_order_acquire) != 0; }

// While a background compile runs, runs go in spans of this many iterations,
// each waited for, so the context can switch kernels between two of them.
constexpr int kPacedSpan = 10;

struct Prof {
    sl_ctx* c;
    int kernel;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    Prof(sl_ctx* c_, int k, cudaStream_t s_ = nullptr) : c(c_), kernel(k), s(s_ ? s_ : c_->stream) {
        if (c->profiling) {
            a = take_event(c);
            cudaEventRecord(a, s);
        }
        c->launches++;
    }
    ~Prof() {
        if (a) {
            cudaEvent_t b = take_event(c);
            cudaEventRecord(b, s);
            c->marks.push_back({kernel, a, b});
        }
    }
};
void drain_marks(sl_ctx* c) {
    cudaStreamSynchronize(c->stream);
    if (c->lstream) cudaStreamSynchronize(c->lstream);
    for (auto& m : c->marks) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, m.a, m.b);
        c->prof_ms[m.kernel] += ms;
        c->prof_n[m.kernel] += 1;
        c->event_pool.push_back(m.a);
        c->event_pool.push_back(m.b);
    }
    c->marks.clear();
}
}  // namespace

static int fail(sl_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    g_err = buf;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? SL_ENOMEM : SL_ECUDA, "%s: %s", \
                        #call, cudaGetErrorString(e_));                                       \
    } while (0)

// The L-sampler autotuner: times one even-locus half-sweep of every chain
// with each candidate -- the generic kernel with 32 lanes per (chain, locus)
// task and with 16 (two tasks per warp), and the specialised kernel when it
// was built for SL_LS_KERNEL_AUTO -- on a copy of the chains' graphs (the
// chains are not touched), and keeps the fastest, as the reference times its
// launch shapes and locus groupings (gpu_lodscores.cc:541-596,
// markov_chain.cc:269-311).  Every candidate draws the same graphs, so the
// choice changes speed only.  Pedigrees of one size class (operations and
// allowed rfunction cells, in steps of 25 and 128) share the timing: the
// first context of a class on a device times, later ones (the members of an
// uneven batch) reuse its choice.  Runs once per context, outside any
// capture, before its first L-sampler work.
static std::mutex g_ls_class_mu;
static std::map<std::tuple<int, int, int, int, int, bool>, int> g_ls_class;

static int ls_tune(sl_ctx* ctx) {
    if (!ctx->ls_tune_pending) return SL_OK;
    ctx->ls_tune_pending = false;
    const ProblemDev& P = ctx->P;
    const bool jit = ctx->jit_ls.kern != nullptr;
    const auto key = std::make_tuple(ctx->device, P.ls_fast, P.K / 25, P.ls_arena / 128, std::min(ctx->n_chains, 64),
                                     jit);
    if (!jit) {
        std::lock_guard<std::mutex> g(g_ls_class_mu);
        auto it = g_ls_class.find(key);
        if (it != g_ls_class.end()) {
            if (it->second != ctx->ls_choice) ++ctx->ls_epoch;
            ctx->ls_choice = it->second;
            return SL_OK;
        }
    }
    const int C = ctx->n_chains;
    const size_t words = (size_t)C * P.M * P.W;
    uint32_t* scratch = nullptr;
    if (cudaMalloc(&scratch, sizeof(uint32_t) * words) != cudaSuccess) {
        cudaGetLastError();
        return SL_OK;   // untimed: the first candidate stays
    }
    int st = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpyAsync(scratch, ctx->d_dg, sizeof(uint32_t) * words, cudaMemcpyDeviceToDevice, ctx->stream));
    cudaEvent_t a = take_event(ctx), b = take_event(ctx);
    std::vector<int> cand = {LS_GEN32, LS_GEN16, LS_GEN8};
    if (jit) cand.push_back(LS_JIT);
    int best = ctx->ls_choice;
    float best_ms = 0.f;
    for (int k : cand) {
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {
            if (rep == 1) CK(cudaEventRecord(a, ctx->stream));
            if (k == LS_JIT)
                CK(jit_ls_launch(ctx->jit_ls, scratch, 0, C, ctx->d_even, (int)ctx->even.size(), nullptr, 0, 0, 1, 0,
                                 nullptr, nullptr, 0, ctx->d_status, P.geno, P.prior_f, P.c_theta_f, ctx->sms,
                                 ctx->stream));
            else
                CK(launch_lsampler(P, scratch, 0, C, ctx->d_even, (int)ctx->even.size(), nullptr, 0, 0, 1, 0,
                                   nullptr, 0, ctx->d_status, ctx->stream, ctx->ls_grid, ctx->ls_wpb, nullptr,
                                   ls_lanes(k)));
            if (rep == 1) {
                CK(cudaEventRecord(b, ctx->stream));
                CK(cudaEventSynchronize(b));
                CK(cudaEventElapsedTime(&ms, a, b));
            }
        }
        ctx->ls_tune_ms[k] = ms;
        if (k == cand[0] || ms < best_ms) {
            best = k;
            best_ms = ms;
        }
    }
    ctx->event_pool.push_back(a);
    ctx->event_pool.push_back(b);
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(scratch);
    CK(cudaMemcpy(ctx->d_status, &st, sizeof(int), cudaMemcpyHostToDevice));   // the timing runs report nothing
    if (best != ctx->ls_choice) ++ctx->ls_epoch;
    ctx->ls_choice = best;
    if (!jit) {
        std::lock_guard<std::mutex> g(g_ls_class_mu);
        g_ls_class[key] = best;
    }
    return SL_OK;
}

template <typename T>
static int dev_alloc(sl_ctx* ctx, T** p, size_t n) {
    void* q = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T));
    if (e != cudaSuccess) return fail(ctx, SL_ENOMEM, "cudaMalloc(%zu bytes): %s", n * sizeof(T), cudaGetErrorString(e));
    ctx->owned.push_back(q);
    *p = (T*)q;
    return SL_OK;
}

template <typename T>
static int upload(sl_ctx* ctx, T** p, const T* host, size_t n) {
    int rc = dev_alloc(ctx, p, n);
    if (rc) return rc;
    if (n) CK(cudaMemcpy(*p, host, n * sizeof(T), cudaMemcpyHostToDevice));
    return SL_OK;
}

// ---------------------------------------------------------------------------
// Host-side tables
// ---------------------------------------------------------------------------

// Per-locus prior of a person's phased state given its genotype code.  The
// reference fills Person::genotypes_prob while parsing, before parents are
// linked, so every person takes the founder branch: the Hardy-Weinberg marker
// probability masked by the typed genotype, then normalised
// (pedigree_parser.cc:157, person.cc:224-299; Snp::init_probs,
// genetic_map.h:68-87).  The sums keep the reference's operand order.
static void build_priors(int M, const double* minor, std::vector<double>& out) {
    out.assign((size_t)M * 16, 0.0);
    for (int l = 0; l < M; ++l) {
        const double mi = minor[l], ma = 1.0 - minor[l];
        double hw[4];
        hw[UU] = ma * ma;
        hw[AU] = mi * ma;
        hw[UA] = mi * ma;
        hw[AA] = mi * mi;
        const double tot = hw[UU] + hw[AU] + hw[UA] + hw[AA];
        for (int v = 0; v < 4; ++v) hw[v] /= tot;
        for (int g = 0; g < 4; ++g) {
            double pr[4];
            for (int v = 0; v < 4; ++v) {
                bool ok = true;
                if (g == G_HETERO) ok = (v == AU || v == UA);
                else if (g == G_HOMOZ_A) ok = (v == UU);
                else if (g == G_HOMOZ_B) ok = (v == AA);
                pr[v] = ok ? hw[v] : 0.0;
            }
            const double t = pr[0] + pr[1] + pr[2] + pr[3];
            for (int v = 0; v < 4; ++v) out[((size_t)l * 4 + g) * 4 + v] = pr[v] / t;
        }
    }
}

// Genotype elimination over phased genotypes {AA=8, AB=4, BA=2, BB=1}
// (elimination.cc:41-183): initial masks from the typed genotypes, then
// homozygote rules repeated until nothing changes.  Returns false when a
// locus has a person with no possible genotype.
namespace {
enum { PG_AA = 8, PG_AB = 4, PG_BA = 2, PG_BB = 1 };
int child_homoz(std::vector<int>& pg, int mother, int father, int child, int homoz) {
    int changes = 0;
    const int other = homoz == PG_AA ? PG_BB : PG_AA;
    if ((pg[child] ^ homoz) == 0) {
        if (pg[mother] & other) { pg[mother] ^= other; ++changes; }
        if (pg[father] & other) { pg[father] ^= other; ++changes; }
    }
    return changes;
}
int parent_homoz(std::vector<int>& pg, int parent, int other_parent, int child, int homoz, int maternal) {
    int changes = 0;
    if ((pg[parent] ^ homoz) == 0) {
        int hetero, other_hetero;
        if ((maternal && homoz == PG_AA) || (!maternal && homoz == PG_BB)) { hetero = PG_AB; other_hetero = PG_BA; }
        else { hetero = PG_BA; other_hetero = PG_AB; }
        const int other_homoz = homoz == PG_AA ? PG_BB : PG_AA;
        if (pg[child] & other_homoz) { pg[child] ^= other_homoz; ++changes; }
        if (pg[child] & other_hetero) { pg[child] ^= other_hetero; ++changes; }
        if ((pg[child] & hetero) && !(pg[child] & homoz)) {
            if (pg[other_parent] & homoz) { pg[other_parent] ^= homoz; ++changes; }
        }
    }
    return changes;
}
}  // namespace

static bool genotype_elimination(const sl_problem_desc* d, std::vector<uint8_t>& legal, int* bad_locus) {
    const int N = d->n_members, M = d->n_markers;
    legal.assign((size_t)M * N, 0);
    std::vector<int> pg(N);
    // phased trait v -> phased genotype bit (genotype.cc:91-102)
    const int bit_of[4] = {PG_AA, PG_BB, PG_BA, PG_AB};
    for (int l = 0; l < M; ++l) {
        for (int j = 0; j < N; ++j) {
            const int g = d->typed[j] ? d->genotypes[(size_t)l * N + j] : G_UNTYPED;
            int m = 15;
            if (g == G_HOMOZ_A) m &= PG_AA;
            else if (g == G_HETERO) m &= (PG_AB | PG_BA);
            else if (g == G_HOMOZ_B) m &= PG_BB;
            pg[j] = m;
        }
        while (true) {
            int changes = 0;
            for (int i = 0; i < N; ++i) {
                if (d->mother[i] < 0) continue;
                const int mat = d->mother[i], pat = d->father[i];
                changes += parent_homoz(pg, mat, pat, i, PG_AA, 1);
                changes += parent_homoz(pg, mat, pat, i, PG_BB, 1);
                changes += parent_homoz(pg, pat, mat, i, PG_AA, 0);
                changes += parent_homoz(pg, pat, mat, i, PG_BB, 0);
                changes += child_homoz(pg, mat, pat, i, PG_AA);
                changes += child_homoz(pg, mat, pat, i, PG_BB);
            }
            for (int i = 0; i < N; ++i)
                if (pg[i] == 0) { *bad_locus = l; return false; }
            if (changes == 0) break;
        }
        for (int j = 0; j < N; ++j) {
            uint8_t m = 0;
            for (int v = 0; v < 4; ++v)
                if (pg[j] & bit_of[v]) m |= (uint8_t)(1u << v);
            legal[(size_t)l * N + j] = m;
        }
    }
    return true;
}

// Trait peel without a descent graph: log P(T) (Peeler::calc_trait_prob,
// peeler.cc:65-73), evaluated once on the host in FP64.
static double host_trait_prob(const sl_problem_desc* d, const std::vector<OpDev>& ops,
                              const std::vector<int32_t>& od, int arena) {
    std::vector<double> A(arena, 0.0);
    auto dig = [](int ext, int pos) { return (ext >> (2 * pos)) & 3; };
    auto phased = [](int m, int p, int i, int j) {
        const int ma = (m == AA) || (m == AU && i == 0) || (m == UA && i == 1);
        const int pa = (p == AA) || (p == AU && j == 0) || (p == UA && j == 1);
        if (ma) return pa ? (int)AA : (int)AU;
        return pa ? (int)UA : (int)UU;
    };
    for (size_t k = 0; k < ops.size(); ++k) {
        const OpDev& op = ops[k];
        const int ncell = 1 << (2 * op.c);
        const double* trait = d->disease_prob + 4 * op.peel;
        for (int cell = 0; cell < ncell; ++cell) {
            bool valid = true;
            for (int q = 0; q < op.c; ++q)
                if (d->disease_prob[4 * od[op.cut_at + q] + dig(cell, q)] == 0.0) valid = false;
            double total = 0.0;
            auto prevs = [&](int ext, double tmp) {
                const int32_t* pd = od.data() + op.prev_at;
                for (int j = 0; j < op.n_prev; ++j) {
                    int idx = 0;
                    for (int q = 0; q < pd[1]; ++q) idx |= dig(ext, pd[2 + q]) << (2 * q);
                    tmp *= A[pd[0] + idx];
                    pd += 2 + pd[1];
                }
                return tmp;
            };
            if (valid) {
                if (op.type == CHILD) {
                    const int mt = dig(cell, op.mpos), pt = dig(cell, op.fpos);
                    for (int i = 0; i < 2; ++i)
                        for (int j = 0; j < 2; ++j) {
                            const int kt = phased(mt, pt, i, j);
                            if (trait[kt] == 0.0) continue;
                            double tmp = prevs(cell | (kt << (2 * op.c)), trait[kt]);
                            tmp *= 0.25;
                            total += tmp;
                        }
                } else if (op.type == PARENT) {
                    for (int a = 0; a < 4; ++a) {
                        if (trait[a] == 0.0) continue;
                        const int ext = cell | (a << (2 * op.c));
                        double tmp = prevs(ext, trait[a]);
                        double cp = 1.0;
                        int mt = a, pt = a;
                        const int32_t* cd = od.data() + op.child_at;
                        for (int c = 0; c < op.n_child; ++c, cd += 4) {
                            const int kt = dig(ext, cd[1]), other = dig(ext, cd[2]);
                            if (cd[3]) pt = other; else mt = other;
                            double ct = 0.0;
                            for (int i = 0; i < 2; ++i)
                                for (int j = 0; j < 2; ++j)
                                    if (phased(mt, pt, i, j) == kt) ct += 0.25;
                            cp *= ct;
                        }
                        tmp *= cp;
                        total += tmp;
                    }
                } else {
                    for (int a = 0; a < 4; ++a) {
                        if (trait[a] == 0.0) continue;
                        total += prevs(cell | (a << (2 * op.c)), trait[a]);
                    }
                }
            }
            A[op.mat_off + cell] = total;
        }
    }
    return std::log(A[ops.back().mat_off]);
}

// The reference's int32 [locus][person][2] graphs <-> the device's packed
// columns: a column's non-founder indicators are the 2 Nnf consecutive int32
// values from offset 2F, so each 32-bit word packs 32 of them in order.
static void pack_columns(const int32_t* src, int N, int F, int W, uint32_t* dst, size_t c0, size_t c1) {
    const int nb = 2 * (N - F);
    for (size_t c = c0; c < c1; ++c) {
        const int32_t* bits = src + (size_t)2 * N * c + 2 * F;
        uint32_t* out = dst + c * W;
        for (int w = 0; w < W; ++w) {
            const int b0 = 32 * w, nbit = std::min(32, nb - b0);
            uint32_t x = 0;
            for (int k = 0; k < nbit; ++k) x |= (uint32_t)(bits[b0 + k] & 1) << k;
            out[w] = x;
        }
    }
}

static void unpack_columns(const uint32_t* src, int N, int F, int W, int32_t* dst, size_t c0, size_t c1) {
    const int nb = 2 * (N - F);
    for (size_t c = c0; c < c1; ++c) {
        int32_t* col = dst + (size_t)2 * N * c;
        std::memset(col, 0, sizeof(int32_t) * 2 * F);
        const uint32_t* in = src + c * W;
        for (int b = 0; b < nb; ++b) col[2 * F + b] = (in[b >> 5] >> (b & 31)) & 1;
    }
}

// Runs f(c0, c1) over [0, n) columns, split across host threads when the
// graphs are large (hundreds of megabytes for 32 chains of a 400-member,
// 10,000-marker pedigree in the reference's layout).
template <typename Fn>
static void for_columns(size_t n, size_t bytes, Fn f) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = bytes < (size_t(8) << 20) ? 1u : std::min<unsigned>(hw, 32u);
    if (nt == 1) {
        f((size_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    const size_t per = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const size_t a = t * per, b = std::min(n, a + per);
        if (a < b) th.emplace_back([=] { f(a, b); });
    }
    for (auto& x : th) x.join();
}

static void pack_graphs(const int32_t* src, int n, int N, int F, int M, int W, uint32_t* dst) {
    for_columns((size_t)n * M, (size_t)n * M * N * 8,
                [&](size_t a, size_t b) { pack_columns(src, N, F, W, dst, a, b); });
}

static void unpack_graphs(const uint32_t* src, int n, int N, int F, int M, int W, int32_t* dst) {
    for_columns((size_t)n * M, (size_t)n * M * N * 8,
                [&](size_t a, size_t b) { unpack_columns(src, N, F, W, dst, a, b); });
}

// Peel-operation descriptors with gather maps: for every previous rfunction,
// the position of each of its keys in this op's (cutset, peel node) index, so
// kernels gather with shifts instead of per-person assignment arrays
// (rfunction.cc:116-142, peel_matrix.h:37-45).
static int build_ops(const sl_problem_desc* d, std::vector<OpDev>& ops, std::vector<int32_t>& od, int& arena,
                     int& max_child) {
    const int N = d->n_members, F = d->n_founders, K = d->n_ops;
    ops.assign(K, OpDev{});
    od.clear();
    arena = 0;
    max_child = 1;
    for (int k = 0; k < K; ++k) {
        OpDev& o = ops[k];
        std::memset(&o, 0, sizeof o);
        o.type = d->op_type[k];
        o.peel = d->op_peelnode[k];
        o.c = d->cutset_off[k + 1] - d->cutset_off[k];
        if (o.type < CHILD || o.type > LAST) return (fail(nullptr, SL_EINVAL, "op %d: bad type %d", k, o.type));
        if (o.peel < 0 || o.peel >= N) return (fail(nullptr, SL_EINVAL, "op %d: bad peel node", k));
        if (o.c > 10) return (fail(nullptr, SL_EINVAL, "op %d: cutset of %d is too large", k, o.c));
        const int32_t* cs = d->cutset + d->cutset_off[k];
        auto pos = [&](int person) {
            if (person == o.peel) return o.c;
            for (int q = 0; q < o.c; ++q)
                if (cs[q] == person) return q;
            return -1;
        };
        o.cut_at = (int)od.size();
        for (int q = 0; q < o.c; ++q) od.push_back(cs[q]);
        o.n_prev = d->prev_off[k + 1] - d->prev_off[k];
        o.prev_at = (int)od.size();
        for (int q = d->prev_off[k]; q < d->prev_off[k + 1]; ++q) {
            const int j = d->prev[q];
            if (j < 0 || j >= k) return (fail(nullptr, SL_EINVAL, "op %d: prev %d is not earlier", k, j));
            const int cj = d->cutset_off[j + 1] - d->cutset_off[j];
            od.push_back(ops[j].mat_off);
            od.push_back(cj);
            for (int r = 0; r < cj; ++r) {
                const int ps = pos(d->cutset[d->cutset_off[j] + r]);
                if (ps < 0) return (fail(nullptr, SL_EINVAL, "op %d: prev %d key outside the cutset", k, j));
                od.push_back(ps);
            }
        }
        o.n_child = d->children_off[k + 1] - d->children_off[k];
        o.child_at = (int)od.size();
        if (o.type == PARENT) {
            for (int q = d->children_off[k]; q < d->children_off[k + 1]; ++q) {
                const int ch = d->children[q];
                if (ch < F || ch >= N) return (fail(nullptr, SL_EINVAL, "op %d: bad child %d", k, ch));
                const bool mum = d->mother[ch] == o.peel;
                const int other = mum ? d->father[ch] : d->mother[ch];
                const int pc = pos(ch), po = pos(other);
                if (pc < 0 || pc >= o.c || po < 0)
                    return (fail(nullptr, SL_EINVAL, "op %d: child %d or its other parent not in the cutset", k, ch));
                od.push_back(ch);
                od.push_back(pc);
                od.push_back(po);
                od.push_back(mum ? 1 : 0);
            }
            max_child = std::max(max_child, o.n_child);
        } else {
            o.n_child = 0;
        }
        if (o.type == CHILD) {
            if (o.peel < F) return (fail(nullptr, SL_EINVAL, "op %d: child peel of a founder", k));
            o.mpos = pos(d->mother[o.peel]);
            o.fpos = pos(d->father[o.peel]);
            if (o.mpos < 0 || o.mpos >= o.c || o.fpos < 0 || o.fpos >= o.c)
                return (fail(nullptr, SL_EINVAL, "op %d: parents of the child not in the cutset", k));
        }
        o.mat_off = arena;
        arena += 1 << (2 * o.c);
        o.prev_ops_at = (int)od.size();
        for (int q = d->prev_off[k]; q < d->prev_off[k + 1]; ++q) od.push_back(d->prev[q]);
    }
    if (ops[K - 1].c != 0) return fail(nullptr, SL_EINVAL, "last op must have an empty cutset");
    if (max_child > 31) return fail(nullptr, SL_EINVAL, "parent peel with %d children", max_child);
    // the FP32 trait peel's scaling targets (LI_SCALE, sl_internal.h): each
    // rfunction by the number of rfunctions its consumer multiplies
    for (int k = 0; k < K; ++k)
        for (int q = d->prev_off[k]; q < d->prev_off[k + 1]; ++q)
            ops[d->prev[q]].scale_to = std::max(0, 120 / std::max(1, ops[k].n_prev) - 4);
    return SL_OK;
}

// ---------------------------------------------------------------------------
// Trait-peel compiler for the batched LOD scorer
// ---------------------------------------------------------------------------
// The trait peel (TraitRfunction::evaluate_*_peel, trait_rfunction.cc:28-137)
// is the same sum-product at every graph, interval and position; only the
// recombination terms differ.  It is compiled once per problem into the
// LI_* program (sl_internal.h): only LOD-valid cells get a slot
// (peel_sequence_generator.cc:155-179), terms whose trait probability is zero
// or that gather an invalid cell are dropped (they add exactly zero in the
// reference), gathers become slot indices, and slots are reused once the op
// that consumes a matrix has run.
namespace {
struct SlotAlloc {
    std::vector<char> used;
    int high = 0;
    bool keep = false;   // never reuse a slot (every forward value stays for an adjoint)
    int alloc(int n) {
        if (n <= 0) return 0;
        int run = 0;
        for (int i = 0; i < (int)used.size(); ++i) {
            run = used[i] ? 0 : run + 1;
            if (run == n) {
                for (int j = i - n + 1; j <= i; ++j) used[j] = 1;
                return i - n + 1;
            }
        }
        const int first = (int)used.size() - run;
        used.resize(first + n, 0);
        for (int j = first; j < first + n; ++j) used[j] = 1;
        high = std::max(high, (int)used.size());
        return first;
    }
    void release(int first, int n) {
        if (keep) return;
        for (int j = first; j < first + n; ++j) used[j] = 0;
    }
};

int phased_trait_host(int m, int p, int i, int j) {
    const int ma = (m == AA) || (m == AU && i == 0) || (m == UA && i == 1);
    const int pa = (p == AA) || (p == AU && j == 0) || (p == UA && j == 1);
    if (ma) return pa ? (int)AA : (int)AU;
    return pa ? (int)UA : (int)UU;
}
}  // namespace

struct LodProgram {
    std::vector<int32_t> words;
    std::vector<float> consts;
    std::vector<double> consts64;   // the same constants unrounded, for host evaluation
    std::vector<int> cperson, cstate;  // the disease probability each constant is
    std::vector<int> starts;        // word offset of every instruction
    int slots = 0;
    int nscale = 0;                 // LI_SCALE instructions
};

// full = true compiles the peel without dropping zero-probability cells or
// terms and without reusing slots: the form the adjoint needs (a zero
// disease probability still has a derivative with respect to the model).
static void compile_lod_program(const sl_problem_desc* d, const std::vector<OpDev>& ops, const std::vector<int32_t>& od,
                                LodProgram& out, bool full = false) {
    const int K = (int)ops.size();
    SlotAlloc sa;
    sa.keep = full;
    std::vector<std::vector<int>> slot_of(K);   // cell -> slot, -1 when not LOD-valid
    std::vector<int> first(K, 0), count(K, 0);
    auto dig = [](int ext, int pos) { return (ext >> (2 * pos)) & 3; };
    auto cnst_ps = [&](int person, int state) {
        const double v = d->disease_prob[4 * person + state];
        out.consts.push_back((float)v);
        out.consts64.push_back(v);
        out.cperson.push_back(person);
        out.cstate.push_back(state);
        return (int)out.consts.size() - 1;
    };
    auto& W = out.words;
    for (int k = 0; k < K; ++k) {
        const OpDev& op = ops[k];
        const int ncell = 1 << (2 * op.c);
        const int32_t* cut = od.data() + op.cut_at;
        const double* trait = d->disease_prob + 4 * op.peel;
        std::vector<int> valid;
        for (int cell = 0; cell < ncell; ++cell) {
            bool ok = true;
            if (!full)
                for (int q = 0; q < op.c; ++q)
                    if (d->disease_prob[4 * cut[q] + dig(cell, q)] == 0.0) ok = false;
            if (ok) valid.push_back(cell);
        }
        // recombination terms of the children this op transmits to
        std::vector<int> kids;
        if (op.type == CHILD) kids.push_back(op.peel);
        if (op.type == PARENT)
            for (int c = 0; c < op.n_child; ++c) kids.push_back(od[op.child_at + 4 * c]);
        std::vector<int> rec_slot(kids.size());
        for (size_t c = 0; c < kids.size(); ++c) rec_slot[c] = sa.alloc(4);
        struct Term { int ci; std::vector<int> f; };
        std::vector<std::vector<Term>> terms(valid.size());
        std::map<std::pair<int, int>, int> sum_slot;   // (child index, mask) -> slot
        std::vector<std::pair<int, int>> sum_order;
        auto gather = [&](int ext, std::vector<int>& f) {
            const int32_t* pd = od.data() + op.prev_at;
            for (int j = 0; j < op.n_prev; ++j) {
                // pd[0] is the previous op's matrix offset; find that op
                int pk = -1;
                for (int q = 0; q < k; ++q)
                    if (ops[q].mat_off == pd[0]) { pk = q; break; }
                int idx = 0;
                for (int q = 0; q < pd[1]; ++q) idx |= dig(ext, pd[2 + q]) << (2 * q);
                const int sl = slot_of[pk][idx];
                if (sl < 0) return false;
                f.push_back(sl);
                pd += 2 + pd[1];
            }
            return true;
        };
        for (size_t vi = 0; vi < valid.size(); ++vi) {
            const int cell = valid[vi];
            if (op.type == CHILD) {
                const int mt = dig(cell, op.mpos), pt = dig(cell, op.fpos);
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) {
                        const int kt = phased_trait_host(mt, pt, i, j);
                        if (trait[kt] == 0.0 && !full) continue;
                        Term t;
                        if (!gather(cell | (kt << (2 * op.c)), t.f)) continue;
                        t.f.push_back(rec_slot[0] + 2 * i + j);
                        t.ci = cnst_ps(op.peel, kt);
                        terms[vi].push_back(t);
                    }
            } else if (op.type == PARENT) {
                for (int a = 0; a < 4; ++a) {
                    if (trait[a] == 0.0 && !full) continue;
                    const int ext = cell | (a << (2 * op.c));
                    Term t;
                    if (!gather(ext, t.f)) continue;
                    int mt = a, pt = a;
                    bool zero = false;
                    for (int c = 0; c < op.n_child; ++c) {
                        const int32_t* cd = od.data() + op.child_at + 4 * c;
                        const int kt = dig(ext, cd[1]), other = dig(ext, cd[2]);
                        if (cd[3]) pt = other; else mt = other;
                        int mask = 0;
                        for (int i = 0; i < 2; ++i)
                            for (int j = 0; j < 2; ++j)
                                if (phased_trait_host(mt, pt, i, j) == kt) mask |= 1 << (2 * i + j);
                        if (mask == 0) { zero = true; break; }
                        if ((mask & (mask - 1)) == 0) {
                            t.f.push_back(rec_slot[c] + __builtin_ctz(mask));
                        } else {
                            auto key = std::make_pair(c, mask);
                            auto it = sum_slot.find(key);
                            if (it == sum_slot.end()) {
                                const int sl = sa.alloc(1);
                                sum_slot[key] = sl;
                                sum_order.push_back(key);
                                t.f.push_back(sl);
                            } else {
                                t.f.push_back(it->second);
                            }
                        }
                    }
                    if (zero) continue;
                    t.ci = cnst_ps(op.peel, a);
                    terms[vi].push_back(t);
                }
            } else {
                for (int a = 0; a < 4; ++a) {
                    if (trait[a] == 0.0 && !full) continue;
                    Term t;
                    if (!gather(cell | (a << (2 * op.c)), t.f)) continue;
                    t.ci = cnst_ps(op.peel, a);
                    terms[vi].push_back(t);
                }
            }
        }
        // outputs
        count[k] = (int)valid.size();
        first[k] = sa.alloc(count[k]);
        slot_of[k].assign(ncell, -1);
        for (size_t vi = 0; vi < valid.size(); ++vi) slot_of[k][valid[vi]] = first[k] + (int)vi;
        // emit
        for (size_t c = 0; c < kids.size(); ++c) {
            out.starts.push_back((int)W.size());
            W.push_back(LI_REC);
            W.push_back(kids[c]);
            W.push_back(rec_slot[c]);
        }
        for (auto& key : sum_order) {
            const int c = key.first, mask = key.second;
            out.starts.push_back((int)W.size());
            W.push_back(LI_SUM);
            W.push_back(sum_slot[key]);
            W.push_back(__builtin_popcount(mask));
            for (int b = 0; b < 4; ++b)
                if (mask & (1 << b)) W.push_back(rec_slot[c] + b);
        }
        for (size_t vi = 0; vi < valid.size(); ++vi) {
            out.starts.push_back((int)W.size());
            W.push_back(LI_CELL);
            W.push_back(first[k] + (int)vi);
            W.push_back((int)terms[vi].size());
            for (auto& t : terms[vi]) {
                W.push_back((int)t.f.size());
                W.push_back(t.ci);
                for (int f : t.f) W.push_back(f);
            }
        }
        if (count[k] > 0) {
            out.starts.push_back((int)W.size());
            out.nscale++;
            W.push_back(LI_SCALE);
            W.push_back(first[k]);
            W.push_back(count[k]);
            W.push_back(full ? 0 : op.scale_to);
        }
        // temporaries and consumed matrices are dead now
        for (size_t c = 0; c < kids.size(); ++c) sa.release(rec_slot[c], 4);
        for (auto& kv : sum_slot) sa.release(kv.second, 1);
        const int32_t* pd = od.data() + op.prev_at;
        for (int j = 0; j < op.n_prev; ++j) {
            for (int q = 0; q < k; ++q)
                if (ops[q].mat_off == pd[0]) { sa.release(first[q], count[q]); break; }
            pd += 2 + pd[1];
        }
    }
    out.starts.push_back((int)W.size());
    W.push_back(LI_END);
    W.push_back(count[K - 1] > 0 ? first[K - 1] : -1);
    out.slots = std::max(1, sa.high);
}

// Derivatives of Person::disease_prob[person][state] with respect to the
// penetrances of HOMO_U, HETERO, HOMO_A and the disease-allele frequency
// (person.cc:85-119; DiseaseModel::get_apriori_prob2 / get_penetrance_prob2,
// disease_model.cc:139-187; autosomal).
static void disease_prob_grad(const sl_problem_desc* d, int person, int state, double* g4) {
    static const int unph[4] = {0, 2, 1, 1};   // UU, AA, AU, UA -> HOMO_U, HOMO_A, HETERO
    const int t = unph[state];
    const double q = d->disease_freq, pen = d->penetrance[t];
    const int a = d->affection[person];
    g4[0] = g4[1] = g4[2] = g4[3] = 0.0;
    if (d->mother[person] < 0) {
        const double prior[3] = {(1.0 - q) * (1.0 - q), q * (1.0 - q), q * q};
        const double dprior[3] = {-2.0 * (1.0 - q), 1.0 - 2.0 * q, 2.0 * q};
        if (a == 2) { g4[t] = prior[t]; g4[3] = dprior[t] * pen; }
        else if (a == 1) { g4[t] = -prior[t]; g4[3] = dprior[t] * (1.0 - pen); }
        else { g4[3] = dprior[t]; }
    } else {
        if (a == 2) g4[t] = 1.0;
        else if (a == 1) g4[t] = -1.0;
    }
}

// Forward and reverse evaluation of a full program in FP64, with each op's
// cells scaled by a power of two (the same scaling the device uses), for one
// graph / interval / position, or for the peel without a graph (dg NULL,
// every recombination term 0.25).  grad: [theta_L, theta_R, pen x3, freq].
static int host_backward(const sl_problem_desc* d, const LodProgram& prog, const int32_t* dg, int locus, int offset,
                         double* grad, double* loglik) {
    const int N = d->n_members, n = d->lod_per_interval;
    double th = 0, an = 0, th2 = 0, an2 = 0;
    if (dg) {
        th = d->partial_theta[locus] * (offset + 1);
        an = 1.0 - th;
        th2 = d->partial_theta[locus] * (n - offset);
        an2 = 1.0 - th2;
    }
    auto bit = [&](int person, int l, int par) { return dg[(size_t)2 * N * l + 2 * person + par] & 1; };
    std::vector<double> A(prog.slots, 0.0), B(prog.slots, 0.0);
    std::vector<int> exps;
    const int32_t* W = prog.words.data();
    int scale = 0, res = -1;
    for (int s : prog.starts) {
        const int32_t* pc = W + s;
        const int op = pc[0];
        if (op == LI_CELL) {
            const int dst = pc[1], nt = pc[2];
            pc += 3;
            double total = 0.0;
            for (int q = 0; q < nt; ++q) {
                const int nf = pc[0];
                double v = prog.consts64[pc[1]];
                pc += 2;
                for (int f = 0; f < nf; ++f) v *= A[pc[f]];
                pc += nf;
                total += v;
            }
            A[dst] = total;
        } else if (op == LI_REC) {
            const int c = pc[1], dst = pc[2];
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) {
                    double r = 1.0;
                    if (dg) {
                        r = (bit(c, locus, 0) == i) ? an : th;
                        r *= (bit(c, locus + 1, 0) == i) ? an2 : th2;
                        r *= (bit(c, locus, 1) == j) ? an : th;
                        r *= (bit(c, locus + 1, 1) == j) ? an2 : th2;
                    }
                    A[dst + 2 * i + j] = 0.25 * r;
                }
        } else if (op == LI_SUM) {
            double v = 0.0;
            for (int q = 0; q < pc[2]; ++q) v += A[pc[3 + q]];
            A[pc[1]] = v;
        } else if (op == LI_SCALE) {
            double mx = 0.0;
            for (int q = 0; q < pc[2]; ++q) mx = std::max(mx, A[pc[1] + q]);
            int e = 0;
            if (mx > 0.0) {
                e = std::ilogb(mx) - pc[3];
                const double f = std::ldexp(1.0, -e);
                for (int q = 0; q < pc[2]; ++q) A[pc[1] + q] *= f;
            }
            exps.push_back(e);
            scale += e;
        } else {
            res = pc[1];
        }
    }
    if (res < 0 || !(A[res] > 0.0)) return fail(nullptr, SL_EZERO, "trait peel gave a likelihood of 0.0 or less");
    if (loglik) *loglik = std::log(A[res]) + scale * std::log(2.0);
    for (int k = 0; k < 6; ++k) grad[k] = 0.0;
    B[res] = 1.0 / A[res];
    int si = (int)exps.size();
    for (int ii = (int)prog.starts.size() - 1; ii >= 0; --ii) {
        const int32_t* pc = W + prog.starts[ii];
        const int op = pc[0];
        if (op == LI_SCALE) {
            const double f = std::ldexp(1.0, -exps[--si]);
            for (int q = 0; q < pc[2]; ++q) B[pc[1] + q] *= f;
        } else if (op == LI_CELL) {
            const int dst = pc[1], nt = pc[2];
            const double g = B[dst];
            pc += 3;
            for (int q = 0; q < nt; ++q) {
                const int nf = pc[0], ci = pc[1];
                const int32_t* fs = pc + 2;
                double prod = 1.0;
                for (int f = 0; f < nf; ++f) prod *= A[fs[f]];
                if (g != 0.0) {
                    double g4[4];
                    if (d->affection) {
                        disease_prob_grad(d, prog.cperson[ci], prog.cstate[ci], g4);
                        for (int k = 0; k < 4; ++k) grad[2 + k] += g * prod * g4[k];
                    }
                    const double c = prog.consts64[ci];
                    for (int f = 0; f < nf; ++f) {
                        double others = c;
                        for (int f2 = 0; f2 < nf; ++f2)
                            if (f2 != f) others *= A[fs[f2]];
                        B[fs[f]] += g * others;
                    }
                }
                pc += 2 + nf;
            }
        } else if (op == LI_SUM) {
            for (int q = 0; q < pc[2]; ++q) B[pc[3 + q]] += B[pc[1]];
        } else if (op == LI_REC && dg) {
            const int c = pc[1], dst = pc[2];
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) {
                    const double gb = B[dst + 2 * i + j];
                    const bool ml = bit(c, locus, 0) == i, mr = bit(c, locus + 1, 0) == i;
                    const bool pl = bit(c, locus, 1) == j, pr = bit(c, locus + 1, 1) == j;
                    const double a = ml ? an : th, b = mr ? an2 : th2, cc = pl ? an : th, dd = pr ? an2 : th2;
                    const double da = ml ? -1.0 : 1.0, db = mr ? -1.0 : 1.0, dc = pl ? -1.0 : 1.0, ddd = pr ? -1.0 : 1.0;
                    grad[0] += gb * 0.25 * (da * b * cc * dd + a * b * dc * dd);
                    grad[1] += gb * 0.25 * (a * db * cc * dd + a * b * cc * ddd);
                }
        }
    }
    return SL_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* sl_version(void) { return "swiftlink_gb300 0.1 (sm_103a)"; }

const char* sl_last_error(const sl_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

int64_t sl_launch_count(const sl_ctx* ctx) { return ctx ? ctx->launches : 0; }

// Each chain's map at its temperature (GeneticMap::set_temperature,
// genetic_map.cc:95-117, the same operations in the same order):
// theta_t = (t theta) + ((1 - t) 0.5), 1 - theta_t, maf_t = (t maf) + ((1 - t) 0.5).
// The L-sampler's priors stay those of temperature 1: the reference caches
// them while parsing (pedigree_parser.cc:157) and set_minor_freq does not
// rebuild them.
static int upload_chain_maps(sl_ctx* ctx) {
    ProblemDev& P = ctx->P;
    const int C = ctx->n_chains, M = P.M;
    std::vector<double> th((size_t)C * (M - 1)), mi((size_t)C * M), lt((size_t)C * (M - 1)), la((size_t)C * (M - 1));
    std::vector<float> thf((size_t)C * (M - 1));
    for (int c = 0; c < C; ++c) {
        const double t = ctx->temps[c];
        for (int i = 0; i < M - 1; ++i) {
            const double v = (t * ctx->theta_h[i]) + ((1 - t) * 0.5);
            th[(size_t)c * (M - 1) + i] = v;
            thf[(size_t)c * (M - 1) + i] = (float)v;
            lt[(size_t)c * (M - 1) + i] = std::log(v);
            la[(size_t)c * (M - 1) + i] = std::log(1.0 - v);
        }
        for (int i = 0; i < M; ++i) mi[(size_t)c * M + i] = (t * ctx->minor_h[i]) + ((1 - t) * 0.5);
    }
    int rc;
    auto put = [&](auto** dst, const auto* src, size_t n) -> int {
        using E = std::remove_const_t<std::remove_reference_t<decltype(*src)>>;
        if (!*dst) {
            E* p = nullptr;
            if ((rc = dev_alloc(ctx, &p, n))) return rc;
            *dst = p;
        }
        if (cudaMemcpy((void*)*dst, src, sizeof(E) * n, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(ctx, SL_ECUDA, "uploading the chains' maps");
        return SL_OK;
    };
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->lstream) CK(cudaStreamSynchronize(ctx->lstream));
    if ((rc = put((double**)&P.c_theta, th.data(), th.size()))) return rc;
    if ((rc = put((float**)&P.c_theta_f, thf.data(), thf.size()))) return rc;
    if ((rc = put((double**)&P.c_minor, mi.data(), mi.size()))) return rc;
    if (!P.c_lfreq) {
        float2* p = nullptr;
        if ((rc = dev_alloc(ctx, &p, (size_t)C * M))) return rc;
        P.c_lfreq = p;
    }
    CK(launch_lfreq(P.c_minor, const_cast<float2*>(P.c_lfreq), (int64_t)C * M, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if ((rc = put((double**)&P.c_log_theta, lt.data(), lt.size()))) return rc;
    if ((rc = put((double**)&P.c_log_itheta, la.data(), la.size()))) return rc;
    if ((rc = put((double**)&P.temp, ctx->temps.data(), ctx->temps.size()))) return rc;
    return SL_OK;
}

void sl_destroy(sl_ctx* ctx) {
    if (!ctx) return;
    if (ctx->ls_thread.joinable()) ctx->ls_thread.join();
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->lstream) cudaStreamSynchronize(ctx->lstream);
    for (auto& m : ctx->marks) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    for (void* p : ctx->owned) cudaFree(p);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->lstream) cudaStreamDestroy(ctx->lstream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    jit_lod_release(&ctx->jit_reg);
    jit_ls_release(&ctx->jit_ls);
    jit_lod_release(&ctx->jit_smem);
    for (AdjJit& j : ctx->adj_jit_v) adj_jit_release(&j);
    if (ctx->ms_graph) cudaGraphExecDestroy(ctx->ms_graph);
    if (ctx->run_graph) cudaGraphExecDestroy(ctx->run_graph);
    if (ctx->mc3_graph) cudaGraphExecDestroy(ctx->mc3_graph);
    for (auto st : ctx->cap_streams) cudaStreamDestroy(st);
    for (auto ev : ctx->cap_events) cudaEventDestroy(ev);
    cudaSetDevice(cur);
    delete ctx;
}

static int plan_adjoint(sl_ctx* ctx);

int sl_create(const sl_problem_desc* d, const sl_options* opt, sl_ctx** out) {
    sl_ctx* ctx = nullptr;
    if (!d || !opt || !out) return fail(ctx, SL_EINVAL, "null argument");
    *out = nullptr;
    const int N = d->n_members, F = d->n_founders, M = d->n_markers, K = d->n_ops, n = d->lod_per_interval;
    if (N < 1 || F < 1 || F >= N || M < 2 || K < 1 || n < 1)
        return fail(ctx, SL_EINVAL, "bad sizes N=%d F=%d M=%d K=%d n=%d", N, F, M, K, n);
    if (N > 32000) return fail(ctx, SL_EINVAL, "pedigree too large (%d members)", N);
    if (d->sex_linked) return fail(ctx, SL_EINVAL, "sex-linked analysis is not supported on the GPU");
    if (opt->n_chains < 1) return fail(ctx, SL_EINVAL, "n_chains must be >= 1");
    if (opt->lod_flags & ~SL_LOD_ZERO_OK) return fail(ctx, SL_EINVAL, "unknown lod_flags %#x", opt->lod_flags);
    if (opt->lod_precision != SL_LOD_FP64 && opt->lod_precision != SL_LOD_FP32_RESCALED &&
        opt->lod_precision != SL_LOD_FP64_RESCALED)
        return fail(ctx, SL_EINVAL, "unknown lod_precision %d", opt->lod_precision);
    if (opt->sampler_precision != SL_SAMPLER_EXACT && opt->sampler_precision != SL_SAMPLER_FAST)
        return fail(ctx, SL_EINVAL, "unknown sampler_precision %d", opt->sampler_precision);
    for (int i = 0; i < N; ++i) {
        const bool founder = d->mother[i] < 0;
        if (founder != (i < F)) return fail(ctx, SL_EINVAL, "persons must be ordered founders first");
        if (!founder && (d->mother[i] >= N || d->father[i] < 0 || d->father[i] >= N))
            return fail(ctx, SL_EINVAL, "person %d has bad parents", i);
    }
    for (int l = 0; l + 1 < M; ++l)
        if (!(d->theta[l] > 0.0 && d->theta[l] < 0.5 + 1e-12))
            return fail(ctx, SL_EINVAL, "theta[%d]=%g out of (0, 0.5]", l, d->theta[l]);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(ctx, SL_ENODEV, "no CUDA device available");
    if (opt->device < 0 || opt->device >= ndev) return fail(ctx, SL_EINVAL, "bad device %d", opt->device);

    ctx = new sl_ctx();
    ctx->device = opt->device;
    ctx->n_chains = opt->n_chains;
    ctx->lod_precision = opt->lod_precision;
    ctx->sampler_precision = opt->sampler_precision;
    int rc = SL_OK;
    auto bail = [&](int code) { sl_destroy(ctx); return code; };
    if (cudaSetDevice(ctx->device) != cudaSuccess) return bail(fail(nullptr, SL_ECUDA, "cudaSetDevice failed"));
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, ctx->device);
    ctx->sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->lstream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(nullptr, SL_ECUDA, "stream creation failed"));

    std::vector<OpDev> ops;
    std::vector<int32_t> od;
    int arena = 0, max_child = 1;
    if ((rc = build_ops(d, ops, od, arena, max_child))) return bail(rc);

    // ---- tables
    build_priors(M, d->minor_freq, ctx->prior_table);
    if (d->legal) {
        ctx->legal.assign(d->legal, d->legal + (size_t)M * N);
    } else {
        int bad = -1;
        if (!genotype_elimination(d, ctx->legal, &bad))
            return bail(fail(nullptr, SL_EINVAL, "genotypes inconsistent at locus %d", bad));
    }
    std::vector<uint8_t> geno((size_t)M * N);
    for (size_t i = 0; i < geno.size(); ++i) {
        const int person = (int)(i % N);
        const int g = d->typed[person] ? (d->genotypes[i] & 3) : 0;
        geno[i] = (uint8_t)(g | (ctx->legal[i] << 4));
    }
    std::vector<int16_t> mo(N), fa(N), order;
    std::vector<uint8_t> typed(N), dmask(N);
    for (int i = 0; i < N; ++i) {
        mo[i] = (int16_t)d->mother[i];
        fa[i] = (int16_t)d->father[i];
        typed[i] = d->typed[i] ? 1 : 0;
        uint8_t m = 0;
        for (int v = 0; v < 4; ++v)
            if (d->disease_prob[4 * i + v] != 0.0) m |= (uint8_t)(1u << v);
        dmask[i] = m;
    }
    {  // parents before children (descent_graph.cc:320-355)
        std::vector<char> vis(N, 0);
        for (int i = 0; i < F; ++i) { order.push_back((int16_t)i); vis[i] = 1; }
        while ((int)order.size() < N) {
            size_t before = order.size();
            for (int i = F; i < N; ++i)
                if (!vis[i] && vis[d->mother[i]] && vis[d->father[i]]) { order.push_back((int16_t)i); vis[i] = 1; }
            if (order.size() == before) return bail(fail(nullptr, SL_EINVAL, "pedigree has a cycle"));
        }
    }
    // generation levels: a person one level below its deeper parent
    std::vector<int16_t> lvl_order;
    std::vector<int32_t> lvl_off;
    {
        std::vector<int> lvl(N, 0);
        int top = 0;
        for (int16_t i : order)
            if (i >= F) {
                lvl[i] = 1 + std::max(lvl[d->mother[i]], lvl[d->father[i]]);
                top = std::max(top, lvl[i]);
            }
        for (int k = 0; k <= top; ++k) {
            lvl_off.push_back((int32_t)lvl_order.size());
            for (int i = 0; i < N; ++i)
                if (lvl[i] == k) lvl_order.push_back((int16_t)i);
        }
        lvl_off.push_back((int32_t)lvl_order.size());
    }
    // non-ignorable meioses (markov_chain.cc:70-80, Person::safe_to_ignore_meiosis person.cc:208-222)
    {
        std::vector<int> nchild(N, 0);
        for (int i = F; i < N; ++i) { nchild[d->mother[i]]++; nchild[d->father[i]]++; }
        for (int m = 0; m < 2 * (N - F); ++m) {
            const int person = F + m / 2;
            const int parent = (m % 2 == 0) ? d->mother[person] : d->father[person];
            const bool ignore = parent < F && nchild[parent] == 1;
            if (!ignore) ctx->meioses.push_back(m);
        }
        if (ctx->meioses.empty()) ctx->meioses.push_back(0);
    }
    for (int l = 0; l < M; ++l) (l % 2 ? ctx->odd : ctx->even).push_back(l);

    ProblemDev& P = ctx->P;
    P.N = N; P.F = F; P.M = M; P.K = K; P.n_lod = n; P.Nnf = N - F;
    P.W = (2 * (N - F) + 31) / 32;
    P.arena = arena;
    // the L-sampler's compact rfunctions (ls_locus, sl_kernels.cu): at a
    // locus, op k's cells number 2^(the sum of its members' rank bits); the
    // warp's arena holds the most any locus needs
    int ls_cap_try = 0;
    {
        auto rank_bits = [](int mask) {
            const int s = __builtin_popcount(mask);
            return s <= 1 ? 0 : (s == 2 ? 1 : 2);
        };
        int most = 1;
        std::vector<int> per_locus(M);
        for (int l = 0; l < M; ++l) {
            const uint8_t* lg = ctx->legal.data() + (size_t)l * N;
            int tot = 0;
            for (int k = 0; k < K; ++k) {
                int b = 0;
                for (int q = 0; q < ops[k].c; ++q) b += rank_bits(lg[od[ops[k].cut_at + q]] & 15);
                tot += 1 << b;
            }
            per_locus[l] = tot;
            most = std::max(most, tot);
        }
        if (most > 65535)   // the tasks' offsets are 16-bit (and such an arena would not fit shared memory)
            return bail(fail(nullptr, SL_EINVAL, "L-sampler needs %d rfunction cells at one locus", most));
        P.ls_arena = most;
        // a task's shared memory holds the cells of 98% of the loci whole (in
        // steps of 32); the few loci that need more put their last rfunctions'
        // cells in the task's slice of a global spill buffer.  Not worth it
        // when it saves less than an eighth of the arena.
        std::sort(per_locus.begin(), per_locus.end());
        int cap = per_locus[(size_t)((M - 1) * 0.98)];
        cap = (cap + 31) / 32 * 32;
        ls_cap_try = (cap < most && most - cap >= most / 8) ? cap : most;
        P.ls_cap = most;
        P.ls_spill_cells = 0;
        P.ls_spill_slots = 0;
        P.ls_spill_chains = 0;
        P.ls_spill = nullptr;
    }
    P.max_child = max_child;
    P.fag_bytes = 0;
    P.marker_trans = std::log(0.5) * (2 * (N - F));
    P.lod_zero_ok = (opt->lod_flags & SL_LOD_ZERO_OK) ? 1 : 0;
    P.ls_fast = opt->sampler_precision == SL_SAMPLER_FAST ? 1 : 0;
    if ((rc = upload(ctx, (int16_t**)&P.mother, mo.data(), N))) return bail(rc);
    if ((rc = upload(ctx, (int16_t**)&P.father, fa.data(), N))) return bail(rc);
    if ((rc = upload(ctx, (uint8_t**)&P.geno, geno.data(), geno.size()))) return bail(rc);
    {   // each locus's typed members for the founder-allele graphs, heterozygotes first
        if (N > 16383) return bail(fail(nullptr, SL_EINVAL, "more than 16383 members"));
        // (every list starts on a 16-byte boundary and is padded to whole 16-byte chunks: the kernel
        // copies it to shared memory with 16-byte asynchronous copies)
        std::vector<int32_t> off(M, 0);
        std::vector<uint16_t> ent, cnt(M), nhet(M);
        ent.reserve((size_t)M * (N + 8));
        for (int l = 0; l < M; ++l) {
            off[l] = (int32_t)ent.size();
            int nh = 0, nt = 0;
            for (int pass = 0; pass < 2; ++pass)
                for (int i = 0; i < N; ++i) {
                    const int g = geno[(size_t)l * N + i] & 3;
                    if (g == G_UNTYPED || (g == G_HETERO) != (pass == 0)) continue;
                    ent.push_back((uint16_t)(i << 2 | g));
                    nh += pass == 0;
                    ++nt;
                }
            while (ent.size() % 8) ent.push_back(0);
            cnt[l] = (uint16_t)nt;
            nhet[l] = (uint16_t)nh;
        }
        if (ent.empty()) ent.assign(8, 0);
        if (ent.size() > (size_t)INT32_MAX) return bail(fail(nullptr, SL_EINVAL, "typed-member lists too long"));
        if ((rc = upload(ctx, (int32_t**)&P.typ_off, off.data(), off.size()))) return bail(rc);
        if ((rc = upload(ctx, (uint16_t**)&P.typ_ent, ent.data(), ent.size()))) return bail(rc);
        if ((rc = upload(ctx, (uint16_t**)&P.typ_cnt, cnt.data(), cnt.size()))) return bail(rc);
        if ((rc = upload(ctx, (uint16_t**)&P.typ_nhet, nhet.data(), nhet.size()))) return bail(rc);
    }
    if ((rc = upload(ctx, (uint8_t**)&P.typed, typed.data(), N))) return bail(rc);
    if ((rc = upload(ctx, (double**)&P.prior, ctx->prior_table.data(), ctx->prior_table.size()))) return bail(rc);
    if ((rc = upload(ctx, (double**)&P.theta, d->theta, M - 1))) return bail(rc);
    if ((rc = upload(ctx, (double**)&P.partial, d->partial_theta, M - 1))) return bail(rc);
    if ((rc = upload(ctx, (double**)&P.minor, d->minor_freq, M))) return bail(rc);
    {   // FP32 and logarithm tables of the fast kernels
        std::vector<float> thf(M - 1), pf(M - 1), prf(ctx->prior_table.size());
        std::vector<double> lt(M - 1), la(M - 1);
        for (int i = 0; i < M - 1; ++i) {
            thf[i] = (float)d->theta[i];
            pf[i] = (float)d->partial_theta[i];
            lt[i] = std::log(d->theta[i]);
            la[i] = std::log(1.0 - d->theta[i]);
        }
        for (size_t i = 0; i < prf.size(); ++i) prf[i] = (float)ctx->prior_table[i];
        if ((rc = upload(ctx, (float**)&P.theta_f, thf.data(), M - 1))) return bail(rc);
        if ((rc = upload(ctx, (float**)&P.partial_f, pf.data(), M - 1))) return bail(rc);
        if ((rc = upload(ctx, (double**)&P.log_theta, lt.data(), M - 1))) return bail(rc);
        if ((rc = upload(ctx, (double**)&P.log_itheta, la.data(), M - 1))) return bail(rc);
        if ((rc = upload(ctx, (float**)&P.prior_f, prf.data(), prf.size()))) return bail(rc);
    }
    if ((rc = upload(ctx, (double**)&P.dprob, d->disease_prob, (size_t)4 * N))) return bail(rc);
    if ((rc = upload(ctx, (uint8_t**)&P.dmask, dmask.data(), N))) return bail(rc);
    if ((rc = upload(ctx, (OpDev**)&P.ops, ops.data(), K))) return bail(rc);
    if ((rc = upload(ctx, (int32_t**)&P.opdata, od.data(), od.size()))) return bail(rc);
    P.opdata_n = (int32_t)od.size();
    // small operation tables are copied to every L-sampler block; large ones
    // (hundreds of members) would take residency from the arenas
    P.ls_stage_ops = K * sizeof(OpDev) + od.size() * 4 <= 16 * 1024 ? 1 : 0;
    if ((rc = upload(ctx, (int16_t**)&P.fag_order, order.data(), N))) return bail(rc);
    if ((rc = upload(ctx, (int16_t**)&P.lvl_order, lvl_order.data(), N))) return bail(rc);
    if ((rc = upload(ctx, (int32_t**)&P.lvl_off, lvl_off.data(), lvl_off.size()))) return bail(rc);
    P.n_lvl = (int32_t)lvl_off.size() - 1;

    // ---- launch shapes from the shared-memory footprint of one task
    const size_t lst = lsampler_smem_shared(P);
    if (ls_cap_try < P.ls_arena) {
        // the split arena only where it keeps a tenth more tasks resident (where
        // registers, not shared memory, bound the residency it would only cost)
        auto wpb_for = [&]() {
            return (int)std::max<size_t>(1, std::min<size_t>(4, (kSmemBudget - lst) / lsampler_smem_per_warp(P)));
        };
        const int whole = lsampler_resident_tasks(P, wpb_for());
        P.ls_cap = ls_cap_try;
        const int split = lsampler_resident_tasks(P, wpb_for());
        if (split * 10 < whole * 11) P.ls_cap = P.ls_arena;
        P.ls_spill_cells = P.ls_arena - P.ls_cap;
    }
    const size_t lsw = lsampler_smem_per_warp(P);
    const size_t lodw = (size_t)arena * (ctx->lod_precision == SL_LOD_FP32_RESCALED ? 4 : 8);
    if (lst + lsw > kSmemBudget || lodw > kSmemBudget)
        return bail(fail(nullptr, SL_EINVAL, "peel sequence needs %zu bytes per task, above the shared-memory budget",
                         std::max(lsw, lodw)));
    ctx->ls_wpb = (int)std::max<size_t>(1, std::min<size_t>(4, (kSmemBudget - lst) / lsw));
    ctx->lod_wpb = (int)std::max<size_t>(1, std::min<size_t>(4, kSmemBudget / lodw));
    const size_t per_sm = prop.sharedMemPerMultiprocessor;
    const int ls_blocks = std::max(1, (int)std::min<size_t>(16, per_sm / (lst + ctx->ls_wpb * lsw + 1024)));
    const int lod_blocks = std::max(1, (int)std::min<size_t>(16, per_sm / (ctx->lod_wpb * lodw + 1024)));
    ctx->ls_grid = ctx->sms * ls_blocks;
    ctx->lod_grid = ctx->sms * lod_blocks;
    if (P.ls_spill_cells > 0) {
        // per chain, one slice per task slot of the largest L-sampler grid:
        // ls_grid blocks of up to max(ls_wpb, 4) tasks (the lane groups pack 1,
        // 2 or 4 tasks per warp)
        P.ls_spill_slots = (int64_t)ctx->ls_grid * std::max(ctx->ls_wpb, 4);
        P.ls_spill_chains = ctx->n_chains;
        const size_t n = (size_t)P.ls_spill_chains * P.ls_spill_slots * P.ls_spill_cells;
        if (P.ls_fast) {
            float* sp = nullptr;
            if ((rc = dev_alloc(ctx, &sp, n))) return bail(rc);
            P.ls_spill = sp;
        } else {
            double* sp = nullptr;
            if ((rc = dev_alloc(ctx, &sp, n))) return bail(rc);
            P.ls_spill = sp;
        }
    }
    // founder-allele-graph block: the size that keeps the most threads resident
    // per SM (a chain-by-locus grid then fits in as few waves as possible)
    ctx->ms_threads = 0;
    {
        int best = 0;
        for (int t = 32; t <= 128; t += 32) {
            const size_t b = fag_smem(N, F, t, ctx->sampler_precision == SL_SAMPLER_FAST) + 1024;
            if (b > kSmemBudget) break;
            const int resident = t * (int)std::min<size_t>(32, per_sm / b);
            if (resident > best) { best = resident; ctx->ms_threads = t; }
        }
    }
    if (!ctx->ms_threads)
        return bail(fail(nullptr, SL_EINVAL, "founder-allele graph state too large for shared memory"));

    // ---- state buffers
    const int C = ctx->n_chains;
    const int64_t npos = (int64_t)(M - 1) * n;
    if ((rc = dev_alloc(ctx, &ctx->d_dg, (size_t)C * M * P.W))) return bail(rc);
    CK(cudaMemset(ctx->d_dg, 0, sizeof(uint32_t) * (size_t)C * M * P.W));
    if ((rc = dev_alloc(ctx, &ctx->d_acc, npos))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_init, npos))) return bail(rc);
    ctx->vals_graphs = std::max(C, 64);
    if ((rc = dev_alloc(ctx, &ctx->d_vals, (size_t)ctx->vals_graphs * npos))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_raw, (size_t)C * 2 * M))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_fb, (size_t)C * 2 * M))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_raw32, (size_t)C * 2 * M))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_badc, C))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_maps, (size_t)C * M))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_mu, (size_t)C * M))) return bail(rc);
    CK(cudaMemset(ctx->d_badc, 0, C));
    if ((rc = dev_alloc(ctx, &ctx->d_status, 1))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_sel, C))) return bail(rc);
    if ((rc = upload(ctx, &ctx->d_even, ctx->even.data(), ctx->even.size()))) return bail(rc);
    if ((rc = upload(ctx, &ctx->d_odd, ctx->odd.data(), ctx->odd.size()))) return bail(rc);
    if ((rc = upload(ctx, &ctx->d_meioses, ctx->meioses.data(), ctx->meioses.size()))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_morder, (size_t)C * ctx->meioses.size()))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_loci, M))) return bail(rc);
    CK(cudaMemset(ctx->d_status, 0, sizeof(int)));
    CK(cudaMemset(ctx->d_acc, 0, sizeof(double) * npos));
    CK(cudaMemset(ctx->d_init, 0, npos));
    ctx->theta_h.assign(d->theta, d->theta + M - 1);
    ctx->minor_h.assign(d->minor_freq, d->minor_freq + M);
    ctx->temps.assign(C, 1.0);
    ctx->swap_accept.assign(std::max(1, C - 1), 0);
    ctx->swap_propose.assign(std::max(1, C - 1), 0);
    if ((rc = dev_alloc(ctx, &ctx->d_swap_acc, ctx->swap_accept.size()))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_swap_prop, ctx->swap_propose.size()))) return bail(rc);
    CK(cudaMemset(ctx->d_swap_acc, 0, sizeof(int64_t) * ctx->swap_accept.size()));
    CK(cudaMemset(ctx->d_swap_prop, 0, sizeof(int64_t) * ctx->swap_propose.size()));
    if ((rc = dev_alloc(ctx, (uint8_t**)&ctx->d_mc3, sizeof(Mc3Dev)))) return bail(rc);
    CK(cudaMemset(ctx->d_mc3, 0, sizeof(Mc3Dev)));
    if ((rc = dev_alloc(ctx, &ctx->d_llfag, (size_t)4 * M))) return bail(rc);
    if ((rc = dev_alloc(ctx, &ctx->d_llrec, (size_t)4 * (M - 1)))) return bail(rc);
    if ((rc = upload_chain_maps(ctx))) return bail(rc);
    ctx->trait_prob = host_trait_prob(d, ops, od, arena);
    // compiled trait peel for the batched LOD form
    P.prog = nullptr;
    P.pconst = nullptr;
    P.prog_slots = 0;
    P.prog_threads = 0;
    if (ctx->lod_precision == SL_LOD_FP32_RESCALED) {
        LodProgram prog;
        compile_lod_program(d, ops, od, prog);
        int S = 0;
        for (int t = 128; t >= 32; t /= 2)
            if ((size_t)t * prog.slots * sizeof(float) <= kSmemBudget / 2) { S = t; break; }
        if (!S && (size_t)32 * prog.slots * sizeof(float) <= kSmemBudget) S = 32;
        if (S) {
            if ((rc = upload(ctx, (int32_t**)&P.prog, prog.words.data(), prog.words.size()))) return bail(rc);
            if ((rc = upload(ctx, (float**)&P.pconst, prog.consts.data(), std::max<size_t>(1, prog.consts.size()))))
                return bail(rc);
            P.prog_slots = prog.slots;
            P.prog_threads = S;
        }
        const int req = opt->lod_kernel;
        if (req < SL_LOD_KERNEL_AUTO || req > SL_LOD_KERNEL_JIT_SMEM)
            return bail(fail(nullptr, SL_EINVAL, "unknown lod_kernel %d", req));
        ctx->lod_kernel_req = req;
        if (req != SL_LOD_KERNEL_INTERP) {
            const JitProgramIn in{prog.words.data(), prog.words.size(), prog.consts.data(), F, M, n,
                                  P.W, N - F, prog.slots, P.marker_trans, P.lod_zero_ok};
            const auto t0 = std::chrono::steady_clock::now();
            std::string log_reg, log_smem;
            int rc_reg = -1, rc_smem = -1;
            // the two forms compile concurrently (NVRTC programs are independent)
            std::thread th([&] {
                cudaSetDevice(ctx->device);
                if (req != SL_LOD_KERNEL_JIT_SMEM) rc_reg = jit_lod_compile(in, 128, false, &ctx->jit_reg, &log_reg);
            });
            if (req != SL_LOD_KERNEL_JIT_REG && S)
                rc_smem = jit_lod_compile(in, S, true, &ctx->jit_smem, &log_smem);
            th.join();
            ctx->jit_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (req == SL_LOD_KERNEL_JIT_REG && rc_reg)
                return bail(fail(nullptr, SL_EINVAL, "specialised LOD kernel (registers) failed: %.300s", log_reg.c_str()));
            if (req == SL_LOD_KERNEL_JIT_SMEM && rc_smem)
                return bail(fail(nullptr, SL_EINVAL, "specialised LOD kernel (shared) failed: %.300s", log_smem.c_str()));
        }
        if (!S && !ctx->jit_reg.kern && !ctx->jit_smem.kern) ctx->lod_kernel_sel = SL_LOD_KERNEL_INTERP;
        else if (req == SL_LOD_KERNEL_AUTO) ctx->lod_kernel_sel = SL_LOD_KERNEL_AUTO;
        else ctx->lod_kernel_sel = req;
    }
    std::string ls_src;
    {   // the FP32 L-sampler specialised to the pedigree, on request
        const int req = opt->ls_kernel;
        if (req != SL_LS_KERNEL_GENERIC && req != SL_LS_KERNEL_SPECIALISED && req != SL_LS_KERNEL_BACKGROUND &&
            req != SL_LS_KERNEL_AUTO && req != SL_LS_KERNEL_GENERIC32 && req != SL_LS_KERNEL_GENERIC16 &&
            req != SL_LS_KERNEL_GENERIC8)
            return bail(fail(nullptr, SL_EINVAL, "unknown ls_kernel %d", req));
        if (req == SL_LS_KERNEL_GENERIC) ctx->ls_tune_pending = true;   // 32, 16 or 8 lanes per task, by timing
        if (req == SL_LS_KERNEL_GENERIC16) ctx->ls_choice = LS_GEN16;
        if (req == SL_LS_KERNEL_GENERIC8) ctx->ls_choice = LS_GEN8;
        if (P.ls_fast && req == SL_LS_KERNEL_BACKGROUND) {
            // the source now (host tables in hand), the compile on a thread started once creation has succeeded
            const JitLsIn in{ops.data(), od.data(), K, N, F, M, P.W, N - F, arena, max_child, d->mother, d->father};
            ctx->ls_warp_bytes = jit_ls_warp_bytes(in);
            ctx->jit_ls_wpb = (int)std::max<size_t>(1, std::min<size_t>(4, kSmemBudget / ctx->ls_warp_bytes));
            ls_src = jit_ls_source(in, ctx->jit_ls_wpb);
        }
        if (P.ls_fast && (req == SL_LS_KERNEL_SPECIALISED || req == SL_LS_KERNEL_AUTO)) {
            const JitLsIn in{ops.data(), od.data(), K, N, F, M, P.W, N - F, arena, max_child, d->mother, d->father};
            ctx->jit_ls_wpb = (int)std::max<size_t>(1, std::min<size_t>(4, kSmemBudget / jit_ls_warp_bytes(in)));
            const auto t0 = std::chrono::steady_clock::now();
            std::string log;
            if (jit_ls_compile(in, ctx->jit_ls_wpb, &ctx->jit_ls, &log)) {
                if (req == SL_LS_KERNEL_SPECIALISED)
                    return bail(fail(nullptr, SL_EINVAL, "specialised L-sampler failed: %.300s", log.c_str()));
                ctx->jit_ls = JitLs{};   // AUTO: the generic kernels, timed
            }
            ctx->jit_ls_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            ctx->ls_choice = ctx->jit_ls.kern ? LS_JIT : LS_GEN32;
            ctx->ls_tune_pending = req == SL_LS_KERNEL_AUTO;
        }
    }
    if (d->affection) {
        bool ok = true;
        for (int k = 0; k < K; ++k) ok &= ops[k].n_prev <= 8;
        if (ok) {
            std::vector<float> dpf(4 * (size_t)N), dgr(16 * (size_t)N);
            for (int i = 0; i < N; ++i)
                for (int v = 0; v < 4; ++v) {
                    double g4[4];
                    disease_prob_grad(d, i, v, g4);
                    dpf[4 * i + v] = (float)d->disease_prob[4 * i + v];
                    for (int q = 0; q < 4; ++q) dgr[16 * i + 4 * v + q] = (float)g4[q];
                }
            AdjDev& D = ctx->adj;
            if ((rc = upload(ctx, (float**)&D.dprob, dpf.data(), dpf.size()))) return bail(rc);
            if ((rc = upload(ctx, (float**)&D.dgrad, dgr.data(), dgr.size()))) return bail(rc);
            ctx->adj_ops = ops;
            ctx->adj_od = od;
            ctx->adj_prev.assign(d->prev_off, d->prev_off + K + 1);
            ctx->adj_prevs.assign(d->prev, d->prev + d->prev_off[K]);
            if ((rc = plan_adjoint(ctx))) return bail(rc);
            ctx->has_adjoint = true;
        }
    }
    if (!ls_src.empty()) {
        ctx->ls_pending.store(1, std::memory_order_relaxed);
        ctx->ls_thread = std::thread([ctx, src = std::move(ls_src)] {
            const auto t0 = std::chrono::steady_clock::now();
            std::shared_ptr<const JitBinary> bin = jit_binary(src, "sl_ls_jit.cu");
            ctx->ls_thread_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            ctx->ls_bin = std::move(bin);
            ctx->ls_pending.store(2, std::memory_order_release);
        });
    }
    *out = ctx;
    return SL_OK;
}

static int check_chains(sl_ctx* ctx, int first, int n) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    if (first < 0 || n < 1 || first + n > ctx->n_chains)
        return fail(ctx, SL_EINVAL, "chains [%d, %d) outside [0, %d)", first, first + n, ctx->n_chains);
    return SL_OK;
}

static int status_to_code(sl_ctx* ctx, int st) {
    switch (st) {
        case ST_OK: return SL_OK;
        case ST_ZERO_LIK: return fail(ctx, SL_EZERO, "likelihood is zero (check the penetrance function)");
        case ST_ILLEGAL_DG: return fail(ctx, SL_EILLEGAL, "illegal descent graph given to a sampler");
        case ST_LOD_NONPOS: return fail(ctx, SL_EZERO, "trait peel gave a likelihood of 0.0 or less");
    }
    return fail(ctx, SL_ECUDA, "unknown device status %d", st);
}

int sl_synchronize(sl_ctx* ctx) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->lstream));
    CK(cudaStreamSynchronize(ctx->stream));
    int st = 0;
    CK(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) {
        CK(cudaMemset(ctx->d_status, 0, sizeof(int)));
        return status_to_code(ctx, st);
    }
    return SL_OK;
}

int sl_device_status(sl_ctx* ctx, int32_t* status) {
    if (!ctx || !status) return fail(ctx, SL_EINVAL, "null argument");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    int st = 0;
    CK(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    *status = st;
    return SL_OK;
}

static int stage_host(sl_ctx* ctx, size_t words) {
    if (words <= ctx->h_stage_words) return SL_OK;
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    ctx->h_stage_words = 0;
    CK(cudaMallocHost((void**)&ctx->h_stage, sizeof(uint32_t) * words));
    ctx->h_stage_words = words;
    return SL_OK;
}

int sl_set_descent_graphs(sl_ctx* ctx, int32_t first, int32_t n, const int32_t* dg) {
    int rc = check_chains(ctx, first, n);
    if (rc) return rc;
    if (!dg) return fail(ctx, SL_EINVAL, "null descent graph");
    const ProblemDev& P = ctx->P;
    const size_t words = (size_t)P.M * P.W;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if ((rc = stage_host(ctx, words * n))) return rc;
    pack_graphs(dg, n, P.N, P.F, P.M, P.W, ctx->h_stage);
    CK(cudaMemcpyAsync(ctx->d_dg + words * first, ctx->h_stage, sizeof(uint32_t) * words * n, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SL_OK;
}

int sl_get_descent_graphs(sl_ctx* ctx, int32_t first, int32_t n, int32_t* dg) {
    int rc = check_chains(ctx, first, n);
    if (rc) return rc;
    if (!dg) return fail(ctx, SL_EINVAL, "null descent graph");
    const ProblemDev& P = ctx->P;
    const size_t words = (size_t)P.M * P.W;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if ((rc = stage_host(ctx, words * n))) return rc;
    CK(cudaMemcpyAsync(ctx->h_stage, ctx->d_dg + words * first, sizeof(uint32_t) * words * n, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    unpack_graphs(ctx->h_stage, n, P.N, P.F, P.M, P.W, dg);
    return SL_OK;
}

int sl_get_trait_priors(sl_ctx* ctx, double* out) {
    if (!ctx || !out) return fail(ctx, SL_EINVAL, "null argument");
    const ProblemDev& P = ctx->P;
    // reconstruct [M][N][4] from the genotype codes the context holds
    std::vector<uint8_t> geno((size_t)P.M * P.N);
    CK(cudaMemcpy(geno.data(), P.geno, geno.size(), cudaMemcpyDeviceToHost));
    for (int l = 0; l < P.M; ++l)
        for (int i = 0; i < P.N; ++i) {
            const int g = geno[(size_t)l * P.N + i] & 3;
            for (int v = 0; v < 4; ++v)
                out[((size_t)l * P.N + i) * 4 + v] = ctx->prior_table[((size_t)l * 4 + g) * 4 + v];
        }
    return SL_OK;
}

int sl_get_legal_masks(sl_ctx* ctx, uint8_t* out) {
    if (!ctx || !out) return fail(ctx, SL_EINVAL, "null argument");
    std::memcpy(out, ctx->legal.data(), ctx->legal.size());
    return SL_OK;
}

static int stage_draws(sl_ctx* ctx, const double* u, size_t n) {
    if (n > ctx->u_cap) {
        if (ctx->d_u) {
            cudaFree(ctx->d_u);
            ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->d_u));
            ctx->d_u = nullptr;
        }
        int rc = dev_alloc(ctx, &ctx->d_u, n);
        if (rc) return rc;
        ctx->u_cap = n;
    }
    CK(cudaMemcpyAsync(ctx->d_u, u, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    return SL_OK;
}

int sl_lsampler_loci(sl_ctx* ctx, int32_t first, int32_t n_chains, const int32_t* loci, int32_t n_loci,
                     const double* u, int64_t ucs, int64_t uls) {
    int rc = check_chains(ctx, first, n_chains);
    if (rc) return rc;
    const ProblemDev& P = ctx->P;
    if (!loci || n_loci < 1 || n_loci > P.M || !u) return fail(ctx, SL_EINVAL, "bad locus list or draws");
    std::vector<int32_t> sorted(loci, loci + n_loci);
    std::sort(sorted.begin(), sorted.end());
    for (int i = 0; i < n_loci; ++i) {
        if (sorted[i] < 0 || sorted[i] >= P.M) return fail(ctx, SL_EINVAL, "locus %d out of range", sorted[i]);
        if (i && sorted[i] - sorted[i - 1] < 2)
            return fail(ctx, SL_EINVAL, "loci %d and %d interfere (adjacent or repeated)", sorted[i - 1], sorted[i]);
    }
    if (uls < P.K + 2 * P.N || ucs < (int64_t)P.M * uls)
        return fail(ctx, SL_EINVAL, "draw strides too small (need locus stride >= K + 2N)");
    CK(cudaSetDevice(ctx->device));
    ls_adopt(ctx);
    if ((rc = ls_tune(ctx))) return rc;
    if ((rc = stage_draws(ctx, u, (size_t)n_chains * ucs))) return rc;
    CK(cudaMemcpyAsync(ctx->d_loci, loci, sizeof(int32_t) * n_loci, cudaMemcpyHostToDevice, ctx->stream));
    { Prof pf_(ctx, SL_KERNEL_LSAMPLER);
      CK(ls_launch(ctx, first, n_chains, ctx->d_loci, n_loci, ctx->d_u, ucs, uls, 0, 0, nullptr, 0,
                       ctx->stream));
    }
    return sl_synchronize(ctx);
}

int sl_lsampler_sweep(sl_ctx* ctx, int32_t first, int32_t n_chains, const double* u, int64_t ucs, int64_t uls) {
    int rc = check_chains(ctx, first, n_chains);
    if (rc) return rc;
    const ProblemDev& P = ctx->P;
    if (!u) return fail(ctx, SL_EINVAL, "null draws");
    if (uls < P.K + 2 * P.N || ucs < (int64_t)P.M * uls)
        return fail(ctx, SL_EINVAL, "draw strides too small (need locus stride >= K + 2N)");
    CK(cudaSetDevice(ctx->device));
    ls_adopt(ctx);
    if ((rc = ls_tune(ctx))) return rc;
    if ((rc = stage_draws(ctx, u, (size_t)n_chains * ucs))) return rc;
    { Prof pf_(ctx, SL_KERNEL_LSAMPLER);
      CK(ls_launch(ctx, first, n_chains, ctx->d_even, (int)ctx->even.size(), ctx->d_u, ucs, uls, 0, 0,
                       nullptr, 0, ctx->stream));
    }
    { Prof pf_(ctx, SL_KERNEL_LSAMPLER);
      CK(ls_launch(ctx, first, n_chains, ctx->d_odd, (int)ctx->odd.size(), ctx->d_u, ucs, uls, 0, 0,
                       nullptr, 0, ctx->stream));
    }
    return sl_synchronize(ctx);
}

int sl_msampler_sweep(sl_ctx* ctx, int32_t first, int32_t n_chains, const int32_t* meioses, int32_t n_meioses,
                      const double* u, int64_t ucs) {
    int rc = check_chains(ctx, first, n_chains);
    if (rc) return rc;
    const ProblemDev& P = ctx->P;
    if (!meioses || n_meioses < 1 || !u) return fail(ctx, SL_EINVAL, "bad meiosis list or draws");
    for (int j = 0; j < n_meioses; ++j)
        if (meioses[j] < 0 || meioses[j] >= 2 * P.Nnf) return fail(ctx, SL_EINVAL, "meiosis %d out of range", meioses[j]);
    if (ucs < (int64_t)n_meioses * P.M) return fail(ctx, SL_EINVAL, "draw stride too small (need n_meioses * M)");
    CK(cudaSetDevice(ctx->device));
    if ((size_t)n_meioses > ctx->mlist_cap) {
        if (ctx->d_mlist) {
            cudaFree(ctx->d_mlist);
            ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->d_mlist));
            ctx->d_mlist = nullptr;
        }
        if ((rc = dev_alloc(ctx, &ctx->d_mlist, n_meioses))) return rc;
        ctx->mlist_cap = n_meioses;
    }
    if ((rc = stage_draws(ctx, u, (size_t)n_chains * ucs))) return rc;
    CK(cudaMemcpyAsync(ctx->d_mlist, meioses, sizeof(int32_t) * n_meioses, cudaMemcpyHostToDevice, ctx->stream));
    { Prof pf_(ctx, SL_KERNEL_MSAMPLER);
      ctx->launches += msweep_kernels(ctx, n_meioses) - 1;   // one counted by Prof
      CK(launch_msampler(P, ctx->d_dg, first, n_chains, ctx->d_mlist, 0, n_meioses, ctx->d_u, ucs, 0, 0, nullptr, 0,
                       ctx->d_raw, ctx->d_raw32, ctx->d_fb, ctx->d_badc, ctx->d_maps, ctx->d_status, ctx->ms_threads,
                       ctx->sampler_precision == SL_SAMPLER_EXACT, ctx->stream, nullptr, ctx->d_mu, msampler_pairs(ctx)));
    }
    return sl_synchronize(ctx);
}

// One launch of the batched scorer's kernel `which` over G graphs, the
// per-position values into vals (the context's buffer unless given).
static cudaError_t launch_lod_kernel(sl_ctx* ctx, int which, const uint32_t* graphs, int G,
                                     double* vals = nullptr) {
    const ProblemDev& P = ctx->P;
    const int64_t npos = (int64_t)(P.M - 1) * P.n_lod;
    if (!vals) vals = ctx->d_vals;
    if (which == SL_LOD_KERNEL_JIT_REG || which == SL_LOD_KERNEL_JIT_SMEM) {
        const JitLod& j = which == SL_LOD_KERNEL_JIT_REG ? ctx->jit_reg : ctx->jit_smem;
        return jit_lod_launch(j, graphs, (int64_t)P.M * P.W, G, vals, ctx->d_status, P.partial_f, P.log_theta,
                              P.log_itheta, npos * G, ctx->sms, ctx->stream);
    }
    return launch_lod(P, ctx->lod_precision, graphs, (int64_t)P.M * P.W, G, vals, ctx->d_status, ctx->stream,
                      ctx->lod_grid, ctx->lod_wpb);
}

// The timed choice of the batched scorer's kernel, on the first batch scored:
// each candidate runs twice on it (the second run timed), the fastest is kept.
static int autotune_lod(sl_ctx* ctx, const uint32_t* graphs, int G) {
    std::vector<int> cand;
    if (ctx->P.prog) cand.push_back(SL_LOD_KERNEL_INTERP);
    if (ctx->jit_reg.kern) cand.push_back(SL_LOD_KERNEL_JIT_REG);
    if (ctx->jit_smem.kern) cand.push_back(SL_LOD_KERNEL_JIT_SMEM);
    if (cand.empty()) cand.push_back(SL_LOD_KERNEL_INTERP);
    int best = cand[0];
    float best_ms = 0.f;
    cudaEvent_t a = take_event(ctx), b = take_event(ctx);
    for (int k : cand) {
        CK(launch_lod_kernel(ctx, k, graphs, G));
        CK(cudaEventRecord(a, ctx->stream));
        CK(launch_lod_kernel(ctx, k, graphs, G));
        CK(cudaEventRecord(b, ctx->stream));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, a, b));
        if (k == cand[0] || ms < best_ms) {
            best = k;
            best_ms = ms;
        }
    }
    ctx->event_pool.push_back(a);
    ctx->event_pool.push_back(b);
    ctx->lod_kernel_sel = best;
    return SL_OK;
}

// Merge the chains' run tables into the context's table, chain by chain in
// chain order (LODscores::merge_results, lod_score.h:98-105), before the table
// is read or scored into.
static int flush_chain_tables(sl_ctx* ctx) {
    if (!ctx->chain_tables_pending) return SL_OK;
    const int64_t npos = (int64_t)(ctx->P.M - 1) * ctx->P.n_lod;
    CK(cudaSetDevice(ctx->device));
    { Prof pf_(ctx, SL_KERNEL_LOD_MERGE);
    CK(launch_chain_merge(ctx->d_acc_c, ctx->d_init_c, ctx->n_chains, npos, ctx->d_acc, ctx->d_init, ctx->stream)); }
    ctx->chain_tables_pending = false;
    return SL_OK;
}

static int score_device_graphs(sl_ctx* ctx, const uint32_t* graphs, int G) {
    const ProblemDev& P = ctx->P;
    const int64_t npos = (int64_t)(P.M - 1) * P.n_lod;
    if (int rc = flush_chain_tables(ctx)) return rc;
    for (int g0 = 0; g0 < G; g0 += ctx->vals_graphs) {
        const int g = std::min(ctx->vals_graphs, G - g0);
        const uint32_t* gr = graphs + (size_t)g0 * P.M * P.W;
        if (ctx->lod_precision == SL_LOD_FP32_RESCALED && ctx->lod_kernel_sel == SL_LOD_KERNEL_AUTO) {
            int rc = autotune_lod(ctx, gr, g);
            if (rc) return rc;
        }
        { Prof pf_(ctx, SL_KERNEL_LOD);
        CK(launch_lod_kernel(ctx, ctx->lod_precision == SL_LOD_FP32_RESCALED ? ctx->lod_kernel_sel
                                                                              : SL_LOD_KERNEL_INTERP,
                             gr, g)); }
        { Prof pf_(ctx, SL_KERNEL_LOD_MERGE);
      CK(launch_lod_merge(ctx->d_vals, g, npos, ctx->d_acc, ctx->d_init, ctx->stream));
    }
    }
    ctx->lod_count += G;
    return SL_OK;
}

int sl_lod_score_chains(sl_ctx* ctx, int32_t first, int32_t n_chains) {
    int rc = check_chains(ctx, first, n_chains);
    if (rc) return rc;
    CK(cudaSetDevice(ctx->device));
    return score_device_graphs(ctx, ctx->d_dg + (size_t)first * ctx->P.M * ctx->P.W, n_chains);
}

int sl_lod_score_graphs(sl_ctx* ctx, int32_t n_graphs, const int32_t* dgs) {
    if (!ctx || n_graphs < 1 || !dgs) return fail(ctx, SL_EINVAL, "bad graph set");
    const ProblemDev& P = ctx->P;
    const size_t words = (size_t)P.M * P.W;
    CK(cudaSetDevice(ctx->device));
    if (n_graphs > ctx->graphs_cap) {
        if (ctx->d_graphs) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->d_graphs);
            ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->d_graphs));
            ctx->d_graphs = nullptr;
        }
        int rc = dev_alloc(ctx, &ctx->d_graphs, words * n_graphs);
        if (rc) return rc;
        ctx->graphs_cap = n_graphs;
    }
    std::vector<uint32_t> buf(words * n_graphs);
    pack_graphs(dgs, n_graphs, P.N, P.F, P.M, P.W, buf.data());
    CK(cudaMemcpyAsync(ctx->d_graphs, buf.data(), sizeof(uint32_t) * words * n_graphs, cudaMemcpyHostToDevice,
                       ctx->stream));
    int rc = score_device_graphs(ctx, ctx->d_graphs, n_graphs);
    if (rc) return rc;
    return sl_synchronize(ctx);
}

int sl_lod_results(sl_ctx* ctx, double* raw, uint64_t* count, double* trait_prob) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    int rc = flush_chain_tables(ctx);
    if (rc) return rc;
    rc = sl_synchronize(ctx);
    if (rc) return rc;
    const int64_t npos = (int64_t)(ctx->P.M - 1) * ctx->P.n_lod;
    if (raw) CK(cudaMemcpy(raw, ctx->d_acc, sizeof(double) * npos, cudaMemcpyDeviceToHost));
    if (count) *count = ctx->lod_count;
    if (trait_prob) *trait_prob = ctx->trait_prob;
    return SL_OK;
}

int sl_lod_reset(sl_ctx* ctx) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    const int64_t npos = (int64_t)(ctx->P.M - 1) * ctx->P.n_lod;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemsetAsync(ctx->d_acc, 0, sizeof(double) * npos, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_init, 0, npos, ctx->stream));
    if (ctx->d_init_c) CK(cudaMemsetAsync(ctx->d_init_c, 0, (size_t)ctx->n_chains * npos, ctx->stream));
    ctx->chain_tables_pending = false;
    ctx->lod_count = 0;
    return sl_synchronize(ctx);
}

static int check_desc(const sl_problem_desc* d) {
    if (!d) return fail(nullptr, SL_EINVAL, "null problem");
    if (d->n_members < 2 || d->n_founders < 1 || d->n_founders >= d->n_members || d->n_markers < 2 || d->n_ops < 1)
        return fail(nullptr, SL_EINVAL, "bad problem sizes");
    return SL_OK;
}

int sl_problem_legal_masks(const sl_problem_desc* d, uint8_t* out) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (!out) return fail(nullptr, SL_EINVAL, "null output");
    std::vector<uint8_t> legal;
    int bad = -1;
    if (!genotype_elimination(d, legal, &bad)) return fail(nullptr, SL_EINVAL, "genotypes inconsistent at locus %d", bad);
    std::memcpy(out, legal.data(), legal.size());
    return SL_OK;
}

int sl_problem_trait_priors(const sl_problem_desc* d, double* out) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (!out) return fail(nullptr, SL_EINVAL, "null output");
    std::vector<double> table;
    build_priors(d->n_markers, d->minor_freq, table);
    const int N = d->n_members;
    for (int l = 0; l < d->n_markers; ++l)
        for (int i = 0; i < N; ++i) {
            const int g = d->typed[i] ? (d->genotypes[(size_t)l * N + i] & 3) : 0;
            for (int v = 0; v < 4; ++v) out[((size_t)l * N + i) * 4 + v] = table[((size_t)l * 4 + g) * 4 + v];
        }
    return SL_OK;
}

int sl_problem_trait_prob(const sl_problem_desc* d, double* out) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (!out) return fail(nullptr, SL_EINVAL, "null output");
    std::vector<OpDev> ops;
    std::vector<int32_t> od;
    int arena = 0, max_child = 1;
    if ((rc = build_ops(d, ops, od, arena, max_child))) return rc;
    *out = host_trait_prob(d, ops, od, arena);
    return SL_OK;
}

}  // extern "C"

namespace sl {
int ctx_view(sl_ctx* ctx, CtxView* v) {
    if (!ctx || !v) return SL_EINVAL;
    v->P = ctx->P;
    v->stream = (void*)ctx->stream;
    v->d_status = ctx->d_status;
    v->device = ctx->device;
    v->lod_precision = ctx->lod_precision;
    v->lod_grid = ctx->lod_grid;
    v->lod_wpb = ctx->lod_wpb;
    return SL_OK;
}
void ctx_fail(sl_ctx* ctx, int code, const char* msg) { fail(ctx, code, "%s", msg); }

// The scorer the context scores with (sl_lod_score_graphs), G graphs' values
// into vals, launched on the context's stream without synchronising: the
// FP64 forms' kernel, or the FP32 form's selected kernel -- where the first
// scoring has not yet timed the candidates, the specialised form with values
// in registers if it was built, else the interpreter (no timing here, so the
// call stays asynchronous).
cudaError_t ctx_launch_lod(sl_ctx* ctx, const uint32_t* graphs, int G, double* vals) {
    int which = SL_LOD_KERNEL_INTERP;
    if (ctx->lod_precision == SL_LOD_FP32_RESCALED) {
        which = ctx->lod_kernel_sel;
        if (which == SL_LOD_KERNEL_AUTO) which = ctx->jit_reg.kern ? SL_LOD_KERNEL_JIT_REG : SL_LOD_KERNEL_INTERP;
    }
    return launch_lod_kernel(ctx, which, graphs, G, vals);
}
}  // namespace sl

extern "C" {

int sl_get_stream(sl_ctx* ctx, void** stream) {
    if (!ctx || !stream) return fail(ctx, SL_EINVAL, "null argument");
    *stream = (void*)ctx->stream;
    return SL_OK;
}

int sl_profile(sl_ctx* ctx, int32_t enable) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    drain_marks(ctx);
    ctx->profiling = enable != 0;
    return SL_OK;
}

int sl_profile_read(sl_ctx* ctx, int32_t kernel, double* total_ms, int64_t* launches) {
    if (!ctx || kernel < 0 || kernel > 4) return fail(ctx, SL_EINVAL, "bad kernel id");
    drain_marks(ctx);
    if (total_ms) *total_ms = ctx->prof_ms[kernel];
    if (launches) *launches = ctx->prof_n[kernel];
    ctx->prof_ms[kernel] = 0.0;
    ctx->prof_n[kernel] = 0;
    return SL_OK;
}

int sl_problem_lod_program_eval(const sl_problem_desc* d, const int32_t* dg, int32_t locus, int32_t offset,
                                double* out) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (!dg || !out || locus < 0 || locus >= d->n_markers - 1 || offset < 0 || offset >= d->lod_per_interval)
        return fail(nullptr, SL_EINVAL, "bad arguments");
    std::vector<OpDev> ops;
    std::vector<int32_t> od;
    int arena = 0, max_child = 1;
    if ((rc = build_ops(d, ops, od, arena, max_child))) return rc;
    LodProgram prog;
    compile_lod_program(d, ops, od, prog);
    const int N = d->n_members, F = d->n_founders, n = d->lod_per_interval;
    const double th = d->partial_theta[locus] * (offset + 1), an = 1.0 - th;
    const double th2 = d->partial_theta[locus] * (n - offset), an2 = 1.0 - th2;
    auto bit = [&](int person, int l, int par) { return dg[(size_t)2 * N * l + 2 * person + par] & 1; };
    std::vector<double> A(prog.slots, 0.0);
    const int32_t* pc = prog.words.data();
    double result = 0.0;
    while (true) {
        const int op = pc[0];
        if (op == LI_CELL) {
            const int dst = pc[1], nt = pc[2];
            pc += 3;
            double total = 0.0;
            for (int q = 0; q < nt; ++q) {
                const int nf = pc[0];
                double v = prog.consts64[pc[1]];
                pc += 2;
                for (int f = 0; f < nf; ++f) v *= A[pc[f]];
                pc += nf;
                total += v;
            }
            A[dst] = total;
        } else if (op == LI_REC) {
            const int c = pc[1], dst = pc[2];
            pc += 3;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) {
                    double r = (bit(c, locus, 0) == i) ? an : th;
                    r *= (bit(c, locus + 1, 0) == i) ? an2 : th2;
                    r *= (bit(c, locus, 1) == j) ? an : th;
                    r *= (bit(c, locus + 1, 1) == j) ? an2 : th2;
                    A[dst + 2 * i + j] = 0.25 * r;
                }
        } else if (op == LI_SUM) {
            const int dst = pc[1], ns = pc[2];
            double v = 0.0;
            for (int q = 0; q < ns; ++q) v += A[pc[3 + q]];
            A[dst] = v;
            pc += 3 + ns;
        } else if (op == LI_SCALE) {
            pc += 4;
        } else {
            result = pc[1] >= 0 ? A[pc[1]] : 0.0;
            break;
        }
    }
    if (!(result > 0.0)) return fail(nullptr, SL_EZERO, "trait peel gave a likelihood of 0.0 or less");
    int cross = 0;
    for (int i = F; i < N; ++i)
        for (int par = 0; par < 2; ++par) cross += bit(i, locus, par) != bit(i, locus + 1, par);
    const double rec = cross * std::log(d->theta[locus]) + (2 * (N - F) - cross) * std::log(1.0 - d->theta[locus]);
    *out = std::log(result) - rec - std::log(0.5) * (2 * (N - F));
    return SL_OK;
}

// The adjoint's gradients come back in chunks of at most kAdjChunkTasks
// tasks (48 bytes each); its working values live in shared memory.
static constexpr int64_t kAdjChunkTasks = int64_t(1) << 22;

static int adjoint_chunk(sl_ctx* ctx, int64_t ntask) {
    const int64_t want = std::max<int64_t>(1, std::min<int64_t>(ntask, kAdjChunkTasks));
    if (want <= ctx->adj_chunk) return SL_OK;
    cudaStreamSynchronize(ctx->stream);
    if (ctx->d_adjG) {
        cudaFree(ctx->d_adjG);
        ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->d_adjG));
        ctx->d_adjG = nullptr;
    }
    ctx->adj_chunk = 0;
    int rc;
    if ((rc = dev_alloc(ctx, &ctx->d_adjG, (size_t)6 * want))) return rc;
    ctx->adj_chunk = want;
    return SL_OK;
}

// Shared bytes per warp the adjoint aims at when it chooses between keeping
// every matrix and recomputing: at most 32 KB keeps seven or more warps on an
// SM; a plan that keeps everything within it is taken as is.
static constexpr size_t kAdjDefaultBudget = 32 * 1024;

// The adjoint's memory plan (AdjDev): store when every matrix and its
// adjoint fit the budget, else the split into contiguous segments of about
// equal cells that needs the least shared memory (matrices read across a
// segment boundary kept, the rest recomputed).
static int plan_adjoint(sl_ctx* ctx) {
    const std::vector<OpDev>& ops = ctx->adj_ops;
    const int K = (int)ops.size();
    std::vector<int> consumer(K, -1);
    for (int k = 0; k < K; ++k)
        for (int q = ctx->adj_prev[k]; q < ctx->adj_prev[k + 1]; ++q) consumer[ctx->adj_prevs[q]] = k;
    std::vector<int64_t> cells(K);
    int64_t total = 0;
    for (int k = 0; k < K; ++k) total += cells[k] = int64_t(1) << (2 * ops[k].c);
    struct Plan {
        std::vector<int32_t> aoff, seg;
        std::vector<uint8_t> keep;
        int64_t half = 0;
        size_t bytes = 0;
    };
    auto make = [&](int nseg) {
        Plan p;
        p.seg.push_back(0);
        int64_t run = 0;
        for (int k = 0; k < K; ++k) {
            run += cells[k];
            if ((int)p.seg.size() < nseg && run * nseg >= total * (int64_t)p.seg.size() && k + 1 < K)
                p.seg.push_back(k + 1);
        }
        p.seg.push_back(K);
        const int ns = (int)p.seg.size() - 1;
        std::vector<int> seg_of(K);
        for (int g = 0; g < ns; ++g)
            for (int k = p.seg[g]; k < p.seg[g + 1]; ++k) seg_of[k] = g;
        p.keep.assign(K, 0);
        int64_t perm = 0;
        p.aoff.assign(K, 0);
        for (int k = 0; k < K; ++k)
            if (ns == 1 || (consumer[k] >= 0 && seg_of[consumer[k]] != seg_of[k])) {
                p.keep[k] = 1;
                p.aoff[k] = (int32_t)perm;
                perm += cells[k];
            }
        int64_t segn = 0;
        for (int g = 0; g < ns; ++g) {
            int64_t o = 0;
            for (int k = p.seg[g]; k < p.seg[g + 1]; ++k)
                if (!p.keep[k]) {
                    p.aoff[k] = (int32_t)(perm + o);
                    o += cells[k];
                }
            segn = std::max(segn, o);
        }
        p.half = perm + segn;
        p.bytes = (size_t)(8 * p.half + 4 * (K + ctx->P.max_child) + 48 * ctx->P.max_child + 15) & ~(size_t)15;
        return p;
    };
    const size_t budget = ctx->adj_budget ? ctx->adj_budget : kAdjDefaultBudget;
    Plan best = make(1);
    if (best.bytes > budget)
        for (int ns = 2; ns <= std::min(K, 64); ++ns) {
            Plan p = make(ns);
            if (best.seg.size() == 2 || p.bytes < best.bytes) best = std::move(p);   // the first split, then smaller
            if (best.bytes <= budget) break;
        }
    if (best.bytes > kSmemBudget)
        return fail(nullptr, SL_EINVAL, "the trait-peel adjoint needs %zu shared bytes per task", best.bytes);
    // the items of every op under this plan's arena offsets (the gathers of
    // TraitRfunction's peel, trait_rfunction.cc:28-137: the peel node's state,
    // each child's matching transmissions, each previous rfunction's cell)
    std::vector<uint32_t> items;
    std::vector<int32_t> item_at(K);
    {
        const std::vector<int32_t>& od = ctx->adj_od;
        auto dig = [](int ext, int pos) { return (ext >> (2 * pos)) & 3; };
        for (int k = 0; k < K; ++k) {
            const OpDev& op = ops[k];
            item_at[k] = (int32_t)items.size();
            const int nw = adj_item_words(op.n_prev, op.n_child);
            const int ncell = 1 << (2 * op.c);
            for (int cell = 0; cell < ncell; ++cell)
                for (int t = 0; t < 4; ++t) {
                    std::vector<uint32_t> w(nw, 0u);
                    int s;
                    if (op.type == CHILD) s = phased_trait_host(dig(cell, op.mpos), dig(cell, op.fpos), t >> 1, t & 1);
                    else s = t;
                    const int ext = cell | (s << (2 * op.c));
                    w[0] = (uint32_t)s;
                    if (op.type == PARENT) {
                        int mt = t, pt = t;
                        for (int c = 0; c < op.n_child; ++c) {
                            const int32_t* cd = od.data() + op.child_at + 4 * c;
                            const int kt = dig(ext, cd[1]), other = dig(ext, cd[2]);
                            if (cd[3]) pt = other; else mt = other;
                            uint32_t mask = 0;
                            for (int i = 0; i < 2; ++i)
                                for (int j = 0; j < 2; ++j)
                                    if (phased_trait_host(mt, pt, i, j) == kt) mask |= 1u << (2 * i + j);
                            if (c < 7) w[0] |= mask << (2 + 4 * c);
                            else w[1 + (op.n_prev + 1) / 2 + (c - 7) / 8] |= mask << (4 * ((c - 7) % 8));
                        }
                    }
                    const int32_t* pd = od.data() + op.prev_at;
                    const int32_t* po = od.data() + op.prev_ops_at;
                    for (int j = 0; j < op.n_prev; ++j) {
                        int idx = 0;
                        for (int q = 0; q < pd[1]; ++q) idx |= dig(ext, pd[2 + q]) << (2 * q);
                        const uint32_t off = (uint32_t)(best.aoff[po[j]] + idx);
                        w[1 + j / 2] |= off << (16 * (j & 1));
                        pd += 2 + pd[1];
                    }
                    items.insert(items.end(), w.begin(), w.end());
                }
        }
    }
    if (best.half > 65535) return fail(nullptr, SL_EINVAL, "the trait-peel adjoint's arena exceeds 16-bit offsets");
    AdjDev& D = ctx->adj;
    int rc;
    for (void* p : {(void*)D.aoff, (void*)D.seg, (void*)D.keep, (void*)D.items, (void*)D.item_at}) {
        if (!p) continue;
        cudaFree(p);
        ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), p));
    }
    D.aoff = D.seg = nullptr;
    D.keep = nullptr;
    D.items = nullptr;
    D.item_at = nullptr;
    if ((rc = upload(ctx, (uint32_t**)&D.items, items.data(), items.size()))) return rc;
    if ((rc = upload(ctx, (int32_t**)&D.item_at, item_at.data(), item_at.size()))) return rc;
    if ((rc = upload(ctx, (int32_t**)&D.aoff, best.aoff.data(), best.aoff.size()))) return rc;
    if ((rc = upload(ctx, (int32_t**)&D.seg, best.seg.data(), best.seg.size()))) return rc;
    if ((rc = upload(ctx, (uint8_t**)&D.keep, best.keep.data(), best.keep.size()))) return rc;
    D.nseg = (int32_t)best.seg.size() - 1;
    D.half = (int32_t)best.half;
    D.warp_bytes = (int32_t)best.bytes;
    return SL_OK;
}

int sl_set_temperatures(sl_ctx* ctx, const double* temps) {
    if (!ctx || !temps) return fail(ctx, SL_EINVAL, "null argument");
    for (int c = 0; c < ctx->n_chains; ++c)
        if (!(temps[c] > 0.0 && temps[c] <= 1.0))
            return fail(ctx, SL_EINVAL, "temperature %g of chain %d outside (0, 1]", temps[c], c);
    CK(cudaSetDevice(ctx->device));
    ctx->temps.assign(temps, temps + ctx->n_chains);
    return upload_chain_maps(ctx);
}

int sl_ls_kernel_info(sl_ctx* ctx, int32_t* kernel, double* compile_ms) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    ls_adopt(ctx);
    if (kernel) *kernel = ctx->jit_ls.kern && ctx->ls_choice == LS_JIT ? SL_LS_KERNEL_SPECIALISED : SL_LS_KERNEL_GENERIC;
    if (compile_ms) *compile_ms = ls_compiling(ctx) ? -1.0 : ctx->jit_ls_ms;
    return SL_OK;
}

int sl_ls_tuning(sl_ctx* ctx, int32_t* lanes, double* times_ms) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    ls_adopt(ctx);
    if (lanes) *lanes = ctx->ls_choice == LS_JIT ? 0 : ls_lanes(ctx->ls_choice);
    if (times_ms) {
        times_ms[0] = ctx->ls_tune_ms[LS_GEN32];
        times_ms[1] = ctx->ls_tune_ms[LS_GEN16];
        times_ms[2] = ctx->ls_tune_ms[LS_GEN8];
        times_ms[3] = ctx->ls_tune_ms[LS_JIT];
    }
    return SL_OK;
}

int sl_lod_kernel_info(sl_ctx* ctx, int32_t* kernel, double* compile_ms) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    if (kernel) *kernel = ctx->lod_precision == SL_LOD_FP32_RESCALED ? ctx->lod_kernel_sel : SL_LOD_KERNEL_INTERP;
    if (compile_ms) *compile_ms = ctx->jit_ms;
    return SL_OK;
}

// The thread form's arena: a column of 2 half floats and K exponents per
// thread, for the blocks of 128 threads that stay resident on every SM,
// within 4 GiB.
static int adjoint_arena(sl_ctx* ctx, int64_t ntask) {
    const int64_t per = (int64_t)8 * ctx->adj.half + 4 * (int64_t)ctx->P.K;
    int64_t thr = std::min<int64_t>((int64_t)ctx->sms * trait_adjoint_thr_blocks() * 128, (int64_t(4) << 30) / per);
    thr = std::min<int64_t>(thr, (ntask + 127) / 128 * 128);
    thr = thr / 128 * 128;
    if (thr < 128) return fail(ctx, SL_ENOMEM, "the trait-peel adjoint's arena needs %lld bytes per thread", (long long)per);
    const size_t bytes = (size_t)thr * per;
    if (ctx->d_adjA && bytes <= ctx->adj_thr_bytes && (size_t)thr * 8 * ctx->adj.half <= ctx->adj_thr_bytes &&
        thr == ctx->adj_thr)
        return SL_OK;
    cudaStreamSynchronize(ctx->stream);
    for (void* p : {(void*)ctx->d_adjA, (void*)ctx->d_adjE}) {
        if (!p) continue;
        cudaFree(p);
        ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), p));
    }
    ctx->d_adjA = nullptr;
    ctx->d_adjE = nullptr;
    ctx->adj_thr = 0;
    ctx->adj_thr_bytes = 0;
    int rc;
    if ((rc = dev_alloc(ctx, &ctx->d_adjA, (size_t)thr * 2 * ctx->adj.half))) return rc;
    if ((rc = dev_alloc(ctx, &ctx->d_adjE, (size_t)thr * ctx->P.K))) return rc;
    ctx->adj_thr = thr;
    ctx->adj_thr_bytes = bytes;
    return SL_OK;
}

// The specialised form: compiled at its first use (NVRTC, sl_adjjit.cc), for
// plans that keep every matrix.  Returns SL_OK with adj_jit_state 1 when it
// can run.
static int adjoint_jit_build(sl_ctx* ctx) {
    if (ctx->adj_jit_state) return SL_OK;
    AdjJitIn in;
    in.ops = ctx->adj_ops.data();
    in.K = (int)ctx->adj_ops.size();
    in.od = ctx->adj_od.data();
    in.F = ctx->P.F;
    in.M = ctx->P.M;
    in.n = ctx->P.n_lod;
    in.W = ctx->P.W;
    for (int v = 0; v < kAdjJitVariants; ++v) {
        in.min_blocks = kAdjJitMinBlocks[v];
        std::string log;
        if (adj_jit_compile(in, &ctx->adj_jit_v[v], &log)) {
            for (AdjJit& j : ctx->adj_jit_v) adj_jit_release(&j);
            ctx->adj_jit_state = -1;
            ctx->adj_jit_log = log;
            return SL_OK;
        }
    }
    ctx->adj_jit_sel = 0;
    ctx->adj_jit_state = 1;
    return SL_OK;
}

// The specialised form keeps every rfunction, in global memory: it runs
// under a plan that keeps everything, and under the default budget (which
// bounds the shared-memory forms) whenever one block's arena slice per SM fits
// its 4 GiB; a budget the caller set rules it out when the plan splits.  Its
// functions write out every cell and term of an operation, so a cutset of
// more than kAdjJitMaxCut members (1,024 cells and more) would make a function
// too large to compile in reasonable time: such peels keep the other forms.
static constexpr int kAdjJitMaxCut = 4;

static bool adjoint_jit_eligible(const sl_ctx* ctx) {
    for (const OpDev& op : ctx->adj_ops)
        if (op.c > kAdjJitMaxCut) return false;
    if (ctx->adj.nseg == 1) return true;
    if (ctx->adj_budget != 0) return false;
    int64_t half = 0;
    for (const OpDev& op : ctx->adj_ops) half += int64_t(1) << (2 * op.c);
    const int64_t per = adj_jit_block_floats((int)half, ctx->P.K) * (int64_t)sizeof(float);
    return per * ctx->sms <= (int64_t(4) << 30);
}

// The specialised form's arena: the blocks that stay resident on every SM
// (fewer for fewer tasks), each with its slice, within 4 GiB.
static int adjoint_jit_arena(sl_ctx* ctx, int64_t ntask, const AdjJit& j) {
    const int64_t per = adj_jit_block_floats(j.half, ctx->P.K) * (int64_t)sizeof(float);
    int64_t blocks = std::min<int64_t>((int64_t)ctx->sms * j.blocks_per_sm,
                                       (ntask + kAdjJitThreads - 1) / kAdjJitThreads);
    blocks = std::min<int64_t>(blocks, (int64_t(4) << 30) / per);
    if (blocks < 1) return fail(ctx, SL_ENOMEM, "the specialised adjoint's arena needs %lld bytes per block", (long long)per);
    if (ctx->d_adjJ && blocks <= ctx->adj_jit_blocks) return SL_OK;
    cudaStreamSynchronize(ctx->stream);
    if (ctx->d_adjJ) {
        cudaFree(ctx->d_adjJ);
        ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->d_adjJ));
        ctx->d_adjJ = nullptr;
        ctx->adj_jit_blocks = 0;
    }
    int rc;
    if ((rc = dev_alloc(ctx, &ctx->d_adjJ, (size_t)(blocks * per / (int64_t)sizeof(float))))) return rc;
    ctx->adj_jit_blocks = blocks;
    return SL_OK;
}

static cudaError_t adjoint_launch(sl_ctx* ctx, int form, const uint32_t* graphs, int64_t words, int64_t t0,
                                  int64_t nt) {
    const ProblemDev& P = ctx->P;
    if (form == SL_ADJOINT_SPECIALISED)
        return adj_jit_launch(ctx->adj_jit_v[ctx->adj_jit_sel], graphs, words, t0, nt, ctx->d_adjG, ctx->d_status, P.partial_f,
                              ctx->d_adjJ, ctx->adj_jit_blocks, ctx->adj.dprob, ctx->adj.dgrad, P.lod_zero_ok,
                              ctx->stream);
    if (form == SL_ADJOINT_THREAD)
        return launch_trait_adjoint_thr(P, ctx->adj, graphs, words, t0, nt, ctx->d_adjG, ctx->d_status, ctx->d_adjA,
                                        ctx->d_adjE, ctx->adj_thr, ctx->stream);
    return launch_trait_adjoint(P, ctx->adj, graphs, words, t0, nt, ctx->d_adjG, ctx->d_status, ctx->stream, ctx->sms);
}

// The first call with graphs times the forms on its first tasks (up to
// 65,536) and keeps the fastest for the context; a form the caller fixed is
// taken as is.
static int adjoint_choose(sl_ctx* ctx, const uint32_t* graphs, int64_t words, int64_t ntask) {
    if (ctx->adj_form) return SL_OK;
    int rc;
    if (ctx->adj_form_req) {
        if (ctx->adj_form_req == SL_ADJOINT_SPECIALISED) {
            if ((rc = adjoint_jit_build(ctx))) return rc;
            if (ctx->adj_jit_state != 1)
                return fail(ctx, SL_EINVAL, "the specialised adjoint did not build: %s", ctx->adj_jit_log.c_str());
            ctx->adj_jit_sel = ctx->adj_jit_req;
        }
        ctx->adj_form = ctx->adj_form_req;
        return SL_OK;
    }
    const int64_t nt = std::min<int64_t>(ntask, 65536);
    std::vector<int> forms = {SL_ADJOINT_WARP, SL_ADJOINT_THREAD};
    if (adjoint_jit_eligible(ctx)) {
        if ((rc = adjoint_jit_build(ctx))) return rc;
        if (ctx->adj_jit_state == 1) forms.push_back(SL_ADJOINT_SPECIALISED);
    }
    if ((rc = adjoint_arena(ctx, nt))) return rc;
    if (ctx->adj_jit_state == 1 && adjoint_jit_eligible(ctx))
        for (const AdjJit& j : ctx->adj_jit_v)
            if ((rc = adjoint_jit_arena(ctx, nt, j))) return rc;
    int st = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    cudaEvent_t a = take_event(ctx), b = take_event(ctx);
    for (int i = 0; i < 3; ++i) ctx->adj_form_ms[i] = 0.0;
    int best = 0;
    for (int form : forms) {
        // the compiled form: each register budget, the faster kept
        const int nv = form == SL_ADJOINT_SPECIALISED ? kAdjJitVariants : 1;
        int best_v = 0;
        for (int v = 0; v < nv; ++v) {
            if (form == SL_ADJOINT_SPECIALISED) ctx->adj_jit_sel = v;
            CK(adjoint_launch(ctx, form, graphs, words, 0, std::min<int64_t>(nt, 1024)));   // warm-up
            CK(cudaEventRecord(a, ctx->stream));
            CK(adjoint_launch(ctx, form, graphs, words, 0, nt));
            CK(cudaEventRecord(b, ctx->stream));
            CK(cudaEventSynchronize(b));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, a, b));
            if (v == 0 || ms < ctx->adj_form_ms[form - 1]) {
                ctx->adj_form_ms[form - 1] = ms;
                best_v = v;
            }
        }
        if (form == SL_ADJOINT_SPECIALISED) ctx->adj_jit_sel = best_v;
        if (!best || ctx->adj_form_ms[form - 1] < ctx->adj_form_ms[best - 1]) best = form;
    }
    ctx->event_pool.push_back(a);
    ctx->event_pool.push_back(b);
    CK(cudaMemcpy(ctx->d_status, &st, sizeof(int), cudaMemcpyHostToDevice));   // the timing runs report nothing
    ctx->adj_form = best;
    return SL_OK;
}

int sl_trait_backward(sl_ctx* ctx, int32_t n_graphs, const int32_t* dgs, double* grad, double* ptrait_grad) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    if (!ctx->has_adjoint)
        return fail(ctx, SL_EINVAL, "no trait-peel adjoint: the problem carries no disease model (affection is NULL) "
                                    "or an op multiplies more than 8 rfunctions");
    if (n_graphs < 0 || (n_graphs > 0 && (!dgs || !grad))) return fail(ctx, SL_EINVAL, "bad graph set");
    const ProblemDev& P = ctx->P;
    const size_t words = (size_t)P.M * P.W;
    const int64_t npos = (int64_t)(P.M - 1) * P.n_lod;
    CK(cudaSetDevice(ctx->device));
    int rc;
    if (ptrait_grad) {
        if ((rc = adjoint_chunk(ctx, 1))) return rc;
        Prof pr(ctx, SL_KERNEL_LOD);
        CK(launch_trait_adjoint(P, ctx->adj, nullptr, 0, 0, 1, ctx->d_adjG, ctx->d_status, ctx->stream, ctx->sms));
        double g6[6];
        CK(cudaMemcpyAsync(g6, ctx->d_adjG, sizeof(g6), cudaMemcpyDeviceToHost, ctx->stream));
        if ((rc = sl_synchronize(ctx))) return rc;
        for (int k = 0; k < 4; ++k) ptrait_grad[k] = g6[2 + k];
    }
    if (n_graphs == 0) return SL_OK;
    if (n_graphs > ctx->graphs_cap) {
        if (ctx->d_graphs) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->d_graphs);
            ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->d_graphs));
            ctx->d_graphs = nullptr;
        }
        if ((rc = dev_alloc(ctx, &ctx->d_graphs, words * n_graphs))) return rc;
        ctx->graphs_cap = n_graphs;
    }
    std::vector<uint32_t> buf(words * n_graphs);
    pack_graphs(dgs, n_graphs, P.N, P.F, P.M, P.W, buf.data());
    CK(cudaMemcpyAsync(ctx->d_graphs, buf.data(), sizeof(uint32_t) * words * n_graphs, cudaMemcpyHostToDevice,
                       ctx->stream));
    const int64_t ntask = npos * n_graphs;
    if ((rc = adjoint_chunk(ctx, ntask))) return rc;
    if ((rc = adjoint_choose(ctx, ctx->d_graphs, (int64_t)words, ntask))) return rc;
    if (ctx->adj_form == SL_ADJOINT_THREAD && (rc = adjoint_arena(ctx, std::min(ctx->adj_chunk, ntask)))) return rc;
    if (ctx->adj_form == SL_ADJOINT_SPECIALISED &&
        (rc = adjoint_jit_arena(ctx, std::min(ctx->adj_chunk, ntask), ctx->adj_jit_v[ctx->adj_jit_sel])))
        return rc;
    for (int64_t t0 = 0; t0 < ntask; t0 += ctx->adj_chunk) {
        const int64_t nt = std::min(ctx->adj_chunk, ntask - t0);
        {
            Prof pr(ctx, SL_KERNEL_LOD);
            CK(adjoint_launch(ctx, ctx->adj_form, ctx->d_graphs, (int64_t)words, t0, nt));
        }
        CK(cudaMemcpyAsync(grad + t0 * 6, ctx->d_adjG, sizeof(double) * 6 * nt, cudaMemcpyDeviceToHost,
                           ctx->stream));
    }
    return sl_synchronize(ctx);
}

int sl_adjoint_memory(sl_ctx* ctx, int64_t bytes_per_task, int32_t* segments, int64_t* used_bytes) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    if (!ctx->has_adjoint)
        return fail(ctx, SL_EINVAL, "no trait-peel adjoint: the problem carries no disease model (affection is NULL) "
                                    "or an op multiplies more than 8 rfunctions");
    if (bytes_per_task < 0) return fail(ctx, SL_EINVAL, "negative memory budget");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->adj_budget = (size_t)bytes_per_task;
    if (int rc = plan_adjoint(ctx)) return fail(ctx, rc, "%s", sl_last_error(nullptr));
    ctx->adj_form = 0;   // timed again under the new plan
    if (ctx->adj_form_req == SL_ADJOINT_SPECIALISED && !adjoint_jit_eligible(ctx))
        ctx->adj_form_req = 0;   // the specialised form keeps every matrix: not under a split plan
    if (segments) *segments = ctx->adj.nseg;
    if (used_bytes) *used_bytes = ctx->adj.warp_bytes;
    return SL_OK;
}

int sl_adjoint_info(sl_ctx* ctx, int32_t* form, double* warp_ms, double* thread_ms, double* specialised_ms) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    if (form) *form = ctx->adj_form;
    if (warp_ms) *warp_ms = ctx->adj_form_ms[0];
    if (thread_ms) *thread_ms = ctx->adj_form_ms[1];
    if (specialised_ms) *specialised_ms = ctx->adj_form_ms[2];
    return SL_OK;
}

int sl_adjoint_set_form(sl_ctx* ctx, int32_t form, int32_t variant) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    if (!ctx->has_adjoint)
        return fail(ctx, SL_EINVAL, "no trait-peel adjoint: the problem carries no disease model (affection is NULL) "
                                    "or an op multiplies more than 8 rfunctions");
    if (form < 0 || form > SL_ADJOINT_SPECIALISED) return fail(ctx, SL_EINVAL, "unknown adjoint form %d", form);
    if (variant < 0 || variant >= kAdjJitVariants) return fail(ctx, SL_EINVAL, "no variant %d", variant);
    ctx->adj_jit_req = variant;
    if (form == SL_ADJOINT_SPECIALISED && !adjoint_jit_eligible(ctx))
        return fail(ctx, SL_EINVAL, "the specialised adjoint is not built for this peel: it keeps every matrix (the "
                                    "memory budget set splits the peel into %d segments) and takes cutsets of at "
                                    "most %d members", ctx->adj.nseg, kAdjJitMaxCut);
    ctx->adj_form_req = form;
    ctx->adj_form = 0;
    return SL_OK;
}

int sl_adjoint_kernel_info(sl_ctx* ctx, int32_t* shapes, int32_t* variant, int32_t* regs, double* compile_ms) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    if (variant) *variant = ctx->adj_jit_state == 1 ? ctx->adj_jit_sel : -1;
    const AdjJit& j = ctx->adj_jit_v[ctx->adj_jit_sel];
    double ms = 0.0;
    for (const AdjJit& v : ctx->adj_jit_v) ms += v.compile_ms;
    if (shapes) *shapes = ctx->adj_jit_state == 1 ? j.shapes : 0;
    if (regs) *regs = ctx->adj_jit_state == 1 ? j.regs : 0;
    if (compile_ms) *compile_ms = ctx->adj_jit_state == 1 ? ms : (ctx->adj_jit_state ? -1.0 : 0.0);
    return SL_OK;
}

int sl_problem_trait_backward_eval(const sl_problem_desc* d, const int32_t* dg, int32_t locus, int32_t offset,
                                   double* grad) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (!grad || (dg && (locus < 0 || locus >= d->n_markers - 1 || offset < 0 || offset >= d->lod_per_interval)))
        return fail(nullptr, SL_EINVAL, "bad arguments");
    std::vector<OpDev> ops;
    std::vector<int32_t> od;
    int arena = 0, max_child = 1;
    if ((rc = build_ops(d, ops, od, arena, max_child))) return rc;
    LodProgram prog;
    compile_lod_program(d, ops, od, prog, true);
    return host_backward(d, prog, dg, locus, offset, grad, nullptr);
}

int sl_problem_lod_source(const sl_problem_desc* d, int32_t shared, int32_t threads, int32_t lod_flags,
                          int32_t compile, char* buf, int64_t cap, int64_t* len, int32_t* slots, double* compile_ms) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (cap < 0 || (cap > 0 && !buf)) return fail(nullptr, SL_EINVAL, "bad buffer");
    if (threads < 32 || threads > 1024 || threads % 32) return fail(nullptr, SL_EINVAL, "bad threads per block %d", threads);
    std::vector<OpDev> ops;
    std::vector<int32_t> od;
    int arena = 0, max_child = 1;
    if ((rc = build_ops(d, ops, od, arena, max_child))) return rc;
    LodProgram prog;
    compile_lod_program(d, ops, od, prog);
    const int N = d->n_members, F = d->n_founders;
    const JitProgramIn in{prog.words.data(), prog.words.size(), prog.consts.data(), F, d->n_markers,
                          d->lod_per_interval, (2 * (N - F) + 31) / 32, N - F, prog.slots,
                          std::log(0.5) * (2 * (N - F)), (lod_flags & SL_LOD_ZERO_OK) ? 1 : 0};
    const std::string src = jit_lod_source(in, threads, shared != 0);
    if (len) *len = (int64_t)src.size();
    if (slots) *slots = prog.slots;
    if (buf && cap > 0) {
        const size_t n = std::min<size_t>(src.size(), (size_t)cap - 1);
        std::memcpy(buf, src.data(), n);
        buf[n] = 0;
    }
    if (compile) {
        const auto t0 = std::chrono::steady_clock::now();
        const std::shared_ptr<const JitBinary> bin = jit_binary(src, shared ? "sl_lod_jit_smem.cu" : "sl_lod_jit_reg.cu");
        if (compile_ms)
            *compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (bin->rc) return fail(nullptr, SL_EINVAL, "the specialised LOD scorer did not compile: %s", bin->log.c_str());
    }
    return SL_OK;
}

int sl_problem_adjoint_source(const sl_problem_desc* d, int32_t variant, int32_t compile, char* buf, int64_t cap,
                              int64_t* len, int32_t* shapes, double* compile_ms) {
    int rc = check_desc(d);
    if (rc) return rc;
    if (cap < 0 || (cap > 0 && !buf)) return fail(nullptr, SL_EINVAL, "bad buffer");
    if (variant < 0 || variant >= kAdjJitVariants) return fail(nullptr, SL_EINVAL, "no variant %d", variant);
    std::vector<OpDev> ops;
    std::vector<int32_t> od;
    int arena = 0, max_child = 1;
    if ((rc = build_ops(d, ops, od, arena, max_child))) return rc;
    AdjJitIn in;
    in.ops = ops.data();
    in.K = (int)ops.size();
    in.od = od.data();
    in.F = d->n_founders;
    in.M = d->n_markers;
    in.n = d->lod_per_interval;
    in.W = (2 * (d->n_members - d->n_founders) + 31) / 32;
    in.min_blocks = kAdjJitMinBlocks[variant];
    int ns = 0, half = 0;
    const std::string src = adj_jit_source(in, &ns, &half);
    if (len) *len = (int64_t)src.size();
    if (shapes) *shapes = ns;
    if (buf && cap > 0) {
        const size_t n = std::min<size_t>(src.size(), (size_t)cap - 1);
        std::memcpy(buf, src.data(), n);
        buf[n] = 0;
    }
    if (compile) {
        const auto t0 = std::chrono::steady_clock::now();
        const std::shared_ptr<const JitBinary> bin = jit_binary(src, "sl_adj_jit.cu");
        if (compile_ms)
            *compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (bin->rc) return fail(nullptr, SL_EINVAL, "the specialised adjoint did not compile: %s", bin->log.c_str());
    }
    return SL_OK;
}

// Philox4x32-10 uniform, the device stream's host twin (the L/M choice of a
// chain's iteration, for counting the run graph's launches).
static double host_philox_u01(uint64_t key, uint64_t c_hi, uint64_t c_lo) {
    uint32_t c0 = (uint32_t)c_lo, c1 = (uint32_t)(c_lo >> 32), c2 = (uint32_t)c_hi, c3 = (uint32_t)(c_hi >> 32);
    uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c1 = lo1;
        c3 = lo0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    const uint64_t hi = c0 >> 5, lo = c1 >> 6;
    return (double)(hi * 67108864ull + lo) * (1.0 / 9007199254740992.0);
}

// Add a conditional node at the current point of a stream capture and make it
// the capture's dependency; its body graphs are returned.
static cudaError_t capture_conditional(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                                       unsigned size, cudaGraph_t* bodies) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* ed = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, &ed, &nd);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = size;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, ed, nd, &p);
    if (e != cudaSuccess) return e;
    for (unsigned i = 0; i < size; ++i) bodies[i] = p.conditional.phGraph_out[i];
    return cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// The body of chain c's WHILE node: choose / shuffle / key, then a SWITCH of
// the L-sweep (0) and the M-sweep (1), an IF that scores the chain into its
// own LOD table, and the step to the next iteration.
static cudaError_t capture_chain_body(sl_ctx* ctx, int c, cudaGraph_t body, cudaGraphConditionalHandle hwhile,
                                      cudaStream_t s1, cudaStream_t s2) {
    const ProblemDev& P = ctx->P;
    const int M = P.M, nm = (int)ctx->meioses.size();
    const int64_t npos = (int64_t)(M - 1) * P.n_lod;
    const bool exact = ctx->sampler_precision == SL_SAMPLER_EXACT;
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    uint64_t* key = ctx->d_keys + 2 * c;
    uint32_t* graph_c = ctx->d_dg + (size_t)c * M * P.W;
    cudaError_t e = cudaStreamBeginCaptureToGraph(s1, body, nullptr, nullptr, 0, mode);
    if (e != cudaSuccess) return e;
    cudaGraph_t g = body;
    cudaGraphConditionalHandle hsw, hscore;
    if ((e = cudaGraphConditionalHandleCreate(&hsw, g, 2, 0)) != cudaSuccess) return e;
    if ((e = cudaGraphConditionalHandleCreate(&hscore, g, 0, 0)) != cudaSuccess) return e;
    if ((e = launch_chain_iter(ctx->d_run, ctx->d_chain_it, c, key, ctx->d_meioses, nm, ctx->d_morder + (size_t)c * nm,
                               P.temp, hsw, hscore, s1)) != cudaSuccess)
        return e;
    cudaGraph_t sw[2];
    if ((e = capture_conditional(s1, hsw, cudaGraphCondTypeSwitch, 2, sw)) != cudaSuccess) return e;
    // L-sweep of chain c
    if ((e = cudaStreamBeginCaptureToGraph(s2, sw[0], nullptr, nullptr, 0, mode)) != cudaSuccess) return e;
    e = ls_launch(ctx, c, 1, ctx->d_even, (int)ctx->even.size(), nullptr, 0, 0, 0, 0, nullptr, 1,
                        s2, key);
    if (e == cudaSuccess)
        e = ls_launch(ctx, c, 1, ctx->d_odd, (int)ctx->odd.size(), nullptr, 0, 0, 0, 0, nullptr, 1,
                            s2, key);
    cudaError_t e2 = cudaStreamEndCapture(s2, &sw[0]);
    if (e != cudaSuccess || (e = e2) != cudaSuccess) return e;
    // M-sweep of chain c
    if ((e = cudaStreamBeginCaptureToGraph(s2, sw[1], nullptr, nullptr, 0, mode)) != cudaSuccess) return e;
    double* raw = exact ? ctx->d_raw + (size_t)c * 2 * M : ctx->d_raw + (size_t)c * M;   // fast: 2M floats
    void* fb = exact ? (void*)((double*)ctx->d_fb + (size_t)c * 2 * M) : (void*)((float*)ctx->d_fb + (size_t)c * 2 * M);
    e = launch_msampler(P, ctx->d_dg, c, 1, ctx->d_morder + (size_t)c * nm, nm, nm, nullptr, 0, 0, 0, nullptr, 0, raw,
                        ctx->d_raw32 + (size_t)c * 2 * M, fb, ctx->d_badc + c, ctx->d_maps + (size_t)c * M,
                        ctx->d_status, ctx->ms_threads, exact ? 1 : 0, s2, key, ctx->d_mu + (size_t)c * M, msampler_pairs(ctx));
    e2 = cudaStreamEndCapture(s2, &sw[1]);
    if (e != cudaSuccess || (e = e2) != cudaSuccess) return e;
    // scoring of chain c into its own table
    cudaGraph_t sc;
    if ((e = capture_conditional(s1, hscore, cudaGraphCondTypeIf, 1, &sc)) != cudaSuccess) return e;
    if ((e = cudaStreamBeginCaptureToGraph(s2, sc, nullptr, nullptr, 0, mode)) != cudaSuccess) return e;
    double* vals = ctx->d_vals + (size_t)c * npos;
    const int which = ctx->lod_precision == SL_LOD_FP32_RESCALED ? ctx->lod_kernel_sel : SL_LOD_KERNEL_INTERP;
    if (which == SL_LOD_KERNEL_JIT_REG || which == SL_LOD_KERNEL_JIT_SMEM) {
        const JitLod& j = which == SL_LOD_KERNEL_JIT_REG ? ctx->jit_reg : ctx->jit_smem;
        e = jit_lod_launch(j, graph_c, (int64_t)M * P.W, 1, vals, ctx->d_status, P.partial_f, P.log_theta, P.log_itheta, npos, ctx->sms, s2);
    } else {
        e = launch_lod(P, ctx->lod_precision, graph_c, (int64_t)M * P.W, 1, vals, ctx->d_status, s2, ctx->lod_grid,
                       ctx->lod_wpb);
    }
    if (e == cudaSuccess)
        e = launch_lod_merge(vals, 1, npos, ctx->d_acc_c + (size_t)c * npos, ctx->d_init_c + (size_t)c * npos, s2);
    e2 = cudaStreamEndCapture(s2, &sc);
    if (e != cudaSuccess || (e = e2) != cudaSuccess) return e;
    if ((e = launch_chain_advance(ctx->d_run, ctx->d_chain_it, c, hwhile, s1)) != cudaSuccess) return e;
    return cudaStreamEndCapture(s1, &body);
}

// The run graph: init -> one WHILE node per chain (in parallel).
// Everything the run graph needs that cannot happen inside a capture:
// buffers, the kernels' shared-memory limits (set by direct launches that do
// nothing), the timed choice of the scoring kernel, capture streams.
static int prepare_run_graph(sl_ctx* ctx) {
    const ProblemDev& P = ctx->P;
    const int C = ctx->n_chains, M = P.M, nm = (int)ctx->meioses.size();
    const int64_t npos = (int64_t)(M - 1) * P.n_lod;
    const bool exact = ctx->sampler_precision == SL_SAMPLER_EXACT;
    int rc;
    if ((rc = ls_tune(ctx))) return rc;
    if (!ctx->d_run && (rc = dev_alloc(ctx, (uint8_t**)&ctx->d_run, sizeof(RunParams)))) return rc;
    if (!ctx->d_chain_it && (rc = dev_alloc(ctx, &ctx->d_chain_it, C))) return rc;
    if (!ctx->d_keys && (rc = dev_alloc(ctx, &ctx->d_keys, 2 * (size_t)C))) return rc;
    if (!ctx->d_acc_c && (rc = dev_alloc(ctx, &ctx->d_acc_c, (size_t)C * npos))) return rc;
    if (!ctx->d_init_c) {
        // the chains' tables start empty; a graph captured again later (a kernel switch)
        // keeps the scores they hold
        if ((rc = dev_alloc(ctx, &ctx->d_init_c, (size_t)C * npos))) return rc;
        CK(cudaMemsetAsync(ctx->d_init_c, 0, (size_t)C * npos, ctx->stream));
    }
    CK(cudaMemsetAsync(ctx->d_keys, 0, sizeof(uint64_t) * 2 * C, ctx->stream));
    // every chain's selector 0 and want = 2: these launches do nothing
    CK(cudaMemsetAsync(ctx->d_sel, 0, (size_t)C, ctx->stream));
    CK(launch_msampler(P, ctx->d_dg, 0, C, ctx->d_morder, nm, 0, nullptr, 0, 0, 0, ctx->d_sel, 2, ctx->d_raw,
                       ctx->d_raw32, ctx->d_fb, ctx->d_badc, ctx->d_maps, ctx->d_status, ctx->ms_threads, exact ? 1 : 0,
                       ctx->stream, ctx->d_keys, ctx->d_mu, msampler_pairs(ctx)));
    CK(ls_launch(ctx, 0, C, ctx->d_even, (int)ctx->even.size(), nullptr, 0, 0, 0, 0, ctx->d_sel, 2,
                       ctx->stream, ctx->d_keys));
    // the scoring kernel is fixed in the graph: time the candidates now if needed
    if (ctx->lod_precision == SL_LOD_FP32_RESCALED && ctx->lod_kernel_sel == SL_LOD_KERNEL_AUTO) {
        int st = 0;
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        if ((rc = autotune_lod(ctx, ctx->d_dg, std::min(C, ctx->vals_graphs)))) return rc;
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(ctx->d_status, &st, sizeof(int), cudaMemcpyHostToDevice));   // the timing runs report nothing
    }
    {   // one direct scoring launch configures the scoring kernel outside the capture
        int st = 0;
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        CK(launch_lod_kernel(ctx, ctx->lod_precision == SL_LOD_FP32_RESCALED ? ctx->lod_kernel_sel
                                                                             : SL_LOD_KERNEL_INTERP,
                             ctx->d_dg, 1));
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(ctx->d_status, &st, sizeof(int), cudaMemcpyHostToDevice));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    while ((int)ctx->cap_streams.size() < 4) {
        cudaStream_t st;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        ctx->cap_streams.push_back(st);
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        ctx->cap_events.push_back(ev);
    }
    return SL_OK;
}

// Capture one context's run nodes at the current point of stream s (which
// is capturing): init -> one WHILE node per chain (in parallel).  The chains'
// LOD tables are merged into the context's when read (flush_chain_tables).
// s1 and s2 capture the bodies.
static cudaError_t capture_run_nodes(sl_ctx* ctx, cudaStream_t s, cudaStream_t s1, cudaStream_t s2,
                                     bool nested = false) {
    const int C = ctx->n_chains;
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return e;
    std::vector<cudaGraphConditionalHandle> hws(C);
    for (int c = 0; c < C; ++c)
        if ((e = cudaGraphConditionalHandleCreate(&hws[c], g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
    if ((e = launch_run_init(ctx->d_run, ctx->d_chain_it, C, s)) != cudaSuccess) return e;
    // inside an outer loop's body the chains' loops are opened again at every pass
    if (nested && (e = launch_cond_set(hws.data(), C, 1u, s)) != cudaSuccess) return e;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if ((e = cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd)) != cudaSuccess) return e;
    const std::vector<cudaGraphNode_t> init_deps(deps, deps + nd);
    std::vector<cudaGraphNode_t> whiles;
    for (int c = 0; c < C; ++c) {
        const cudaGraphConditionalHandle hw = hws[c];
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = hw;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t wn;
        if ((e = cudaGraphAddNode(&wn, g, init_deps.data(), nullptr, init_deps.size(), &p)) != cudaSuccess) return e;
        whiles.push_back(wn);
        if ((e = capture_chain_body(ctx, c, p.conditional.phGraph_out[0], hw, s1, s2)) != cudaSuccess) return e;
    }
    // the chains' tables stay apart across launches (merged when results are read), so a
    // run split over several calls accumulates every chain's scores as one call does
    return cudaStreamUpdateCaptureDependencies(s, whiles.data(), nullptr, whiles.size(),
                                               cudaStreamSetCaptureDependencies);
}

static int build_run_graph(sl_ctx* ctx) {
    int rc = prepare_run_graph(ctx);
    if (rc) return rc;
    ctx->run_graph_epoch = ctx->ls_epoch;
    cudaStream_t s0 = ctx->cap_streams[0], s1 = ctx->cap_streams[1], s2 = ctx->cap_streams[2];
    cudaGraph_t top = nullptr;
    CK(cudaGraphCreate(&top, 0));
    cudaError_t e = cudaStreamBeginCaptureToGraph(s0, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = capture_run_nodes(ctx, s0, s1, s2);
    cudaError_t e2 = cudaStreamEndCapture(s0, &top);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->run_graph, top, 0);
    cudaGraphDestroy(top);
    if (e != cudaSuccess) {
        ctx->run_graph = nullptr;
        cudaGetLastError();
        return fail(ctx, SL_ECUDA, "capturing the run graph: %s", cudaGetErrorString(e));
    }
    return SL_OK;
}

// The body of an MC3 run's outer WHILE node, captured on stream s: the
// spurt's bounds, the run nodes, the exchange (more than one chain) and the
// step to the next spurt; `set` makes this context's step decide whether the
// loop runs again.
static cudaError_t capture_mc3_spurt(sl_ctx* ctx, cudaStream_t s, cudaGraphConditionalHandle h, int set) {
    cudaError_t e = launch_mc3_begin(ctx->d_mc3, ctx->d_run, s);
    if (e != cudaSuccess) return e;
    if ((e = capture_run_nodes(ctx, s, ctx->cap_streams[1], ctx->cap_streams[2], true)) != cudaSuccess) return e;
    if (ctx->n_chains > 1 &&
        (e = launch_mc3_exchange(ctx->P, ctx->d_mc3, ctx->d_run, 0, ctx->n_chains, ctx->d_dg, ctx->d_llfag,
                                 ctx->d_llrec, ctx->d_swap_acc, ctx->d_swap_prop, s)) != cudaSuccess)
        return e;
    return launch_mc3_end(ctx->d_mc3, ctx->d_run, h, set, s);
}

// Open an outer WHILE node (default 1) at the current point of stream s's
// capture and begin capturing its body on stream sb.
static cudaError_t begin_outer_while(cudaStream_t s, cudaStream_t sb, cudaGraphConditionalHandle* h) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return e;
    if ((e = cudaGraphConditionalHandleCreate(h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
    cudaGraph_t body;
    if ((e = capture_conditional(s, *h, cudaGraphCondTypeWhile, 1, &body)) != cudaSuccess) return e;
    return cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
}

// Instantiate the graph captured on stream s (the capture ends here in any case).
static cudaError_t end_capture(cudaStream_t s, cudaGraph_t top, cudaError_t e, cudaGraphExec_t* out) {
    cudaError_t e2 = cudaStreamEndCapture(s, &top);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, top, 0);
    if (top) cudaGraphDestroy(top);
    if (e != cudaSuccess) {
        *out = nullptr;
        cudaGetLastError();
    }
    return e;
}

// An MC3 run as one launch: WHILE (spurts left) { spurt bounds -> run nodes ->
// exchange -> next spurt }.  Mc3::run's loop (mc3.cc:117-158) on the device.
static int build_mc3_graph(sl_ctx* ctx) {
    int rc = prepare_run_graph(ctx);
    if (rc) return rc;
    ctx->mc3_graph_epoch = ctx->ls_epoch;
    cudaStream_t s0 = ctx->cap_streams[0], sb = ctx->cap_streams[3];
    cudaGraph_t top = nullptr;
    CK(cudaGraphCreate(&top, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaStreamBeginCaptureToGraph(s0, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        e = begin_outer_while(s0, sb, &h);
        if (e == cudaSuccess) {
            e = capture_mc3_spurt(ctx, sb, h, 1);
            cudaGraph_t body = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(sb, &body);
            if (e == cudaSuccess) e = e2;
        }
    }
    if ((e = end_capture(s0, top, e, &ctx->mc3_graph)) != cudaSuccess)
        return fail(ctx, SL_ECUDA, "capturing the MC3 graph: %s", cudaGetErrorString(e));
    return SL_OK;
}

// Drop a context's run graphs captured before its L-sampler kernel changed.
static void drop_stale_graphs(sl_ctx* ctx) {
    if ((ctx->run_graph && ctx->run_graph_epoch != ctx->ls_epoch) ||
        (ctx->mc3_graph && ctx->mc3_graph_epoch != ctx->ls_epoch))
        cudaStreamSynchronize(ctx->stream);   // no launch of them in flight
    if (ctx->run_graph && ctx->run_graph_epoch != ctx->ls_epoch) {
        cudaGraphExecDestroy(ctx->run_graph);
        ctx->run_graph = nullptr;
    }
    if (ctx->mc3_graph && ctx->mc3_graph_epoch != ctx->ls_epoch) {
        cudaGraphExecDestroy(ctx->mc3_graph);
        ctx->mc3_graph = nullptr;
    }
}

// log P(G, graph) from its parts in the reference's order: the interval sums
// added from 0.0 (_recombination_prob), marker transmission first
// (_transmission_prob), then the log of every locus's founder-allele-graph
// likelihood (_sum_prior_prob), joined by log_product (descent_graph.cc:184-269,
// logarithms.cc:27-29).
static double loglik_from_parts(const double* fag, const double* rec, int M, double marker_trans) {
    const double LOG_ZERO = -DBL_MAX;
    double r = 0.0;
    for (int l = 0; l < M - 1; ++l) r += rec[l];
    const double trans = marker_trans + r;
    double prior = 0.0;
    for (int l = 0; l < M; ++l) {
        if (fag[l] == 0.0) { prior = LOG_ZERO; break; }
        prior += std::log(fag[l]);
    }
    return (trans == LOG_ZERO || prior == LOG_ZERO) ? LOG_ZERO : trans + prior;
}

static int loglik_pairs(sl_ctx* ctx, const int* g, const int* t, int npair, double* out) {
    const ProblemDev& P = ctx->P;
    const int M = P.M;
    int g4[4] = {0, 0, 0, 0}, t4[4] = {0, 0, 0, 0};
    for (int k = 0; k < npair; ++k) { g4[k] = g[k]; t4[k] = t[k]; }
    { Prof pf_(ctx, SL_KERNEL_OTHER);
    CK(launch_loglik_parts(P, ctx->d_dg, g4, t4, npair, ctx->d_llfag, ctx->d_llrec, ctx->stream)); }
    std::vector<double> fag((size_t)npair * M), rec((size_t)npair * (M - 1));
    CK(cudaMemcpyAsync(fag.data(), ctx->d_llfag, sizeof(double) * fag.size(), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(rec.data(), ctx->d_llrec, sizeof(double) * rec.size(), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < npair; ++k)
        out[k] = loglik_from_parts(fag.data() + (size_t)k * M, rec.data() + (size_t)k * (M - 1), M, P.marker_trans);
    return SL_OK;
}

// The MC3 exchange after a spurt ending at iteration `it_end` (mc3.cc:138-157),
// queued on the context's stream: a uniformly chosen adjacent pair (r, r+1)
// swaps graphs with probability min(1, exp((xy + yx) - (xx + yy))).  Both
// uniforms come from the Philox stream (stage 9, the spurt's end iteration,
// draws 0 and 1).  The same kernels run inside the persistent MC3 graph.
static int mc3_exchange(sl_ctx* ctx, const sl_run_options* o, int it_end) {
    Mc3Dev m{};
    m.next = it_end;
    m.total = (int64_t)o->burnin + o->iterations;
    m.period = o->exchange_period;
    m.seed = o->seed;
    CK(cudaMemcpyAsync(ctx->d_mc3, &m, sizeof(m), cudaMemcpyHostToDevice, ctx->stream));
    { Prof pf_(ctx, SL_KERNEL_OTHER);
    CK(launch_mc3_exchange(ctx->P, ctx->d_mc3, nullptr, it_end, ctx->n_chains, ctx->d_dg, ctx->d_llfag, ctx->d_llrec,
                           ctx->d_swap_acc, ctx->d_swap_prop, ctx->stream)); }
    ctx->launches += 4;
    return SL_OK;
}

static int scored_chains(const sl_ctx* ctx) {
    int n = 0;
    for (double t : ctx->temps) n += t == 1.0;
    return n;
}

// Score the chains at temperature 1 (runs of consecutive chains per call).
static int score_cold_chains(sl_ctx* ctx) {
    const int C = ctx->n_chains;
    for (int c = 0; c < C;) {
        if (ctx->temps[c] != 1.0) { ++c; continue; }
        int e = c;
        while (e < C && ctx->temps[e] == 1.0) ++e;
        int rc = score_device_graphs(ctx, ctx->d_dg + (size_t)c * ctx->P.M * ctx->P.W, e - c);
        if (rc) return rc;
        c = e;
    }
    return SL_OK;
}

// Capture the device-driven M-sweep once: for every chain c a branch
// memset -> founder-allele graphs (reset) -> [graphs, filter] x nm over that
// chain alone (first = c, one chain); kernels of chains that chose the
// L-sampler return at once.  Seed and iteration come from d_key.
static int build_ms_graph(sl_ctx* ctx) {
    const ProblemDev& P = ctx->P;
    const int C = ctx->n_chains, nm = (int)ctx->meioses.size(), M = P.M;
    const bool exact = ctx->sampler_precision == SL_SAMPLER_EXACT;
    int rc;
    if (!ctx->d_key && (rc = dev_alloc(ctx, &ctx->d_key, 2))) return rc;
    // a first direct launch configures the kernels' shared-memory limits outside the
    // capture; with every chain's selector 0 and want = 2 its kernels do nothing
    CK(cudaMemsetAsync(ctx->d_sel, 0, (size_t)C, ctx->stream));
    CK(launch_set_key(ctx->d_key, 0, 0, ctx->stream));
    CK(launch_msampler(P, ctx->d_dg, 0, C, ctx->d_morder, nm, 0, nullptr, 0, 0, 0, ctx->d_sel, 2, ctx->d_raw,
                       ctx->d_raw32, ctx->d_fb, ctx->d_badc, ctx->d_maps, ctx->d_status, ctx->ms_threads, exact ? 1 : 0,
                       ctx->stream, ctx->d_key, ctx->d_mu, msampler_pairs(ctx)));
    CK(cudaStreamSynchronize(ctx->stream));
    while ((int)ctx->cap_streams.size() < C + 1) {
        cudaStream_t st;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        ctx->cap_streams.push_back(st);
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        ctx->cap_events.push_back(ev);
    }
    cudaStream_t s0 = ctx->cap_streams[C];
    CK(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaEventRecord(ctx->cap_events[C], s0);
    for (int c = 0; c < C && err == cudaSuccess; ++c) {
        cudaStream_t sc = ctx->cap_streams[c];
        err = cudaStreamWaitEvent(sc, ctx->cap_events[C], 0);
        if (err != cudaSuccess) break;
        double* raw = exact ? ctx->d_raw + (size_t)c * 2 * M : ctx->d_raw + (size_t)c * M;   // fast: 2M floats
        void* fb = exact ? (void*)((double*)ctx->d_fb + (size_t)c * 2 * M) : (void*)((float*)ctx->d_fb + (size_t)c * 2 * M);
        err = launch_msampler(P, ctx->d_dg, c, 1, ctx->d_morder + (size_t)c * nm, nm, nm, nullptr, 0, 0, 0,
                              ctx->d_sel + c, 0, raw, ctx->d_raw32 + (size_t)c * 2 * M, fb, ctx->d_badc + c,
                              ctx->d_maps + (size_t)c * M, ctx->d_status, ctx->ms_threads, exact ? 1 : 0, sc,
                              ctx->d_key, ctx->d_mu + (size_t)c * M, msampler_pairs(ctx));
        if (err != cudaSuccess) break;
        err = cudaEventRecord(ctx->cap_events[c], sc);
        if (err != cudaSuccess) break;
        err = cudaStreamWaitEvent(s0, ctx->cap_events[c], 0);
    }
    cudaGraph_t graph = nullptr;
    cudaError_t err2 = cudaStreamEndCapture(s0, &graph);
    if (err == cudaSuccess) err = err2;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&ctx->ms_graph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (err != cudaSuccess) {
        ctx->ms_graph = nullptr;
        return fail(ctx, SL_ECUDA, "capturing the M-sweep graph: %s", cudaGetErrorString(err));
    }
    ctx->ms_graph_kernels = (int64_t)C * msweep_kernels(ctx, nm);
    return SL_OK;
}

// The host's tally of a run-graph span: scored graphs and kernel launches
// (the L/M choices replayed with the same Philox draws).
static void account_span(sl_ctx* ctx, const sl_run_options* o, int first, int end) {
    const int C = ctx->n_chains, nm = (int)ctx->meioses.size();
    const int cold = scored_chains(ctx);
    int64_t kernels = 1;   // init
    for (int it = first; it < end; ++it) {
        const bool score = it >= o->burnin && it % o->scoring_period == 0;
        if (score) {
            ctx->lod_count += (uint64_t)cold;
            ctx->chain_tables_pending = true;
        }
        for (int c = 0; c < C; ++c) {
            const uint64_t hi = ((uint64_t)c << 40) ^ ((uint64_t)it << 4) ^ 7u;
            const bool is_l = host_philox_u01(o->seed, hi, 0) < o->lsampler_prob;
            kernels += 2 + (is_l ? 2 : msweep_kernels(ctx, nm)) + (score && ctx->temps[c] == 1.0 ? 2 : 0);
        }
    }
    ctx->launches += kernels;
}

// Iterations [first, end) of a run: one launch of the run graph, or with
// profiling on the same kernels launched one by one with per-class marks.
static int run_span(sl_ctx* ctx, const sl_run_options* o, int first, int end) {
    const int C = ctx->n_chains;
    const int nm = (int)ctx->meioses.size();
    if (!ctx->profiling) {
        drop_stale_graphs(ctx);
        if (!ctx->run_graph) {
            int rc = build_run_graph(ctx);
            if (rc) return rc;
        }
        const RunParams rp{first, end, o->burnin, o->scoring_period, o->lsampler_prob, o->seed};
        CK(cudaMemcpyAsync(ctx->d_run, &rp, sizeof(rp), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaGraphLaunch(ctx->run_graph, ctx->stream));
        account_span(ctx, o, first, end);
        return SL_OK;
    }
    if (!ctx->ms_graph) {
        int rc = build_ms_graph(ctx);
        if (rc) return rc;
    }
    for (int it = first; it < end; ++it) {
        const uint64_t iter = (uint64_t)it;
        { Prof pf_(ctx, SL_KERNEL_OTHER);
            CK(launch_choose(0, C, o->seed, iter, o->lsampler_prob, ctx->d_sel, ctx->stream)); }
        { Prof pf_(ctx, SL_KERNEL_OTHER);
            CK(launch_shuffle(ctx->d_meioses, nm, ctx->d_morder, 0, C, o->seed, iter, ctx->stream)); }
        // L-sweeps of the chains that chose L run on the second stream while the
        // M-sweeps of the others run here: the two sets of chains are disjoint
        CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->lstream, ctx->ev_fork, 0));
        { Prof pf_(ctx, SL_KERNEL_LSAMPLER, ctx->lstream);
            CK(ls_launch(ctx, 0, C, ctx->d_even, (int)ctx->even.size(), nullptr, 0, 0, o->seed, iter,
                               ctx->d_sel, 1, ctx->lstream)); }
        { Prof pf_(ctx, SL_KERNEL_LSAMPLER, ctx->lstream);
            CK(ls_launch(ctx, 0, C, ctx->d_odd, (int)ctx->odd.size(), nullptr, 0, 0, o->seed, iter,
                               ctx->d_sel, 1, ctx->lstream)); }
        { Prof pf_(ctx, SL_KERNEL_MSAMPLER);
            CK(launch_set_key(ctx->d_key, o->seed, iter, ctx->stream));
            CK(cudaGraphLaunch(ctx->ms_graph, ctx->stream));
            ctx->launches += ctx->ms_graph_kernels; }
        CK(cudaEventRecord(ctx->ev_join, ctx->lstream));
        CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
        if (it >= o->burnin && it % o->scoring_period == 0) {
            int rc = score_cold_chains(ctx);
            if (rc) return rc;
        }
    }
    return SL_OK;
}

// Before a launch of an MC3 graph: the run's parameters and exchange state
// on the context's stream, and the host's tally of the spurts it runs.
static int launch_mc3_run(sl_ctx* ctx, const sl_run_options* o) {
    const int64_t total = (int64_t)o->burnin + o->iterations;
    const RunParams rp{o->first_iteration, o->first_iteration, o->burnin, o->scoring_period, o->lsampler_prob, o->seed};
    Mc3Dev m{};
    m.next = o->first_iteration;
    m.total = total;
    m.period = o->exchange_period;
    m.seed = o->seed;
    CK(cudaMemcpyAsync(ctx->d_run, &rp, sizeof(rp), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->d_mc3, &m, sizeof(m), cudaMemcpyHostToDevice, ctx->stream));
    const int P = o->exchange_period;
    for (int it0 = o->first_iteration; it0 < total;) {
        const int it1 = (int)std::min<int64_t>(total, (it0 / P + 1) * (int64_t)P);
        account_span(ctx, o, it0, it1);
        ctx->launches += 2 + (ctx->n_chains + 63) / 64 + (ctx->n_chains > 1 ? 4 : 0);   // bounds, opens, exchange
        it0 = it1;
    }
    return SL_OK;
}

int sl_run(sl_ctx* ctx, const sl_run_options* o) {
    if (!ctx || !o) return fail(ctx, SL_EINVAL, "null argument");
    if (o->iterations < 0 || o->burnin < 0 || o->scoring_period < 1 || o->first_iteration < 0 ||
        o->exchange_period < 0 || !(o->lsampler_prob >= 0.0 && o->lsampler_prob <= 1.0))
        return fail(ctx, SL_EINVAL, "bad run options");
    CK(cudaSetDevice(ctx->device));
    const int C = ctx->n_chains;
    const int total = o->burnin + o->iterations;
    if (o->first_iteration >= total) return SL_OK;
    ls_adopt(ctx);
    const bool mc3 = o->exchange_period > 0 && C >= 2;
    if (!mc3 && !ls_compiling(ctx)) return run_span(ctx, o, o->first_iteration, total);
    if (mc3 && !ls_compiling(ctx) && !ctx->profiling) {
        // every spurt and exchange in one launch
        drop_stale_graphs(ctx);
        if (!ctx->mc3_graph) {
            int rc = build_mc3_graph(ctx);
            if (rc) return rc;
        }
        int rc = launch_mc3_run(ctx, o);
        if (rc) return rc;
        CK(cudaGraphLaunch(ctx->mc3_graph, ctx->stream));
        return SL_OK;
    }
    // MC3: spurts of exchange_period iterations, each followed by an exchange
    // (Mc3::run, mc3.cc:117-158; iterations are numbered consecutively).  Spurts
    // end at multiples of exchange_period counted from iteration 0, so a run
    // resumed at any first_iteration exchanges where an unbroken run does.
    // While the specialised L-sampler compiles, spans are short and waited for;
    // a run split anywhere gives the same graphs and scores.
    const int P = o->exchange_period;
    for (int it0 = o->first_iteration; it0 < total;) {
        int it1 = mc3 ? std::min(total, (it0 / P + 1) * P) : total;
        const bool paced = ls_compiling(ctx);
        if (paced) it1 = std::min(it1, it0 + kPacedSpan);
        int rc = run_span(ctx, o, it0, it1);
        if (rc) return rc;
        if (paced) {
            CK(cudaStreamSynchronize(ctx->stream));
            ls_adopt(ctx);
        }
        if (mc3 && it1 % P == 0 && (rc = mc3_exchange(ctx, o, it1))) return rc;
        it0 = it1;
    }
    return SL_OK;
}


// ---------------------------------------------------------------------------
// Batches: several contexts (pedigrees of any sizes, each with its chains)
// run by one graph launch per spurt.
// ---------------------------------------------------------------------------
struct sl_batch {
    std::vector<sl_ctx*> ctxs;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> fork;
    std::vector<cudaEvent_t> evs;
    cudaEvent_t ev_root = nullptr, ev_done = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<int> ls_epochs;   // each context's L-sampler kernel switches when the graph was captured
    // MC3 runs: every spurt and exchange of every context in one launch
    cudaStream_t body = nullptr;  // captures the outer loop's body
    cudaGraphExec_t mc3_graph = nullptr;
    std::vector<int> mc3_epochs;
};

void sl_batch_destroy(sl_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->mc3_graph) cudaGraphExecDestroy(b->mc3_graph);
    if (b->body) cudaStreamDestroy(b->body);
    for (auto st : b->fork) cudaStreamDestroy(st);
    for (auto ev : b->evs) cudaEventDestroy(ev);
    if (b->ev_root) cudaEventDestroy(b->ev_root);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int sl_batch_create(sl_ctx* const* ctxs, int32_t n, sl_batch** out) {
    if (!ctxs || n < 1 || !out) return fail(nullptr, SL_EINVAL, "bad batch");
    *out = nullptr;
    for (int j = 0; j < n; ++j) {
        if (!ctxs[j]) return fail(nullptr, SL_EINVAL, "null context %d in batch", j);
        if (ctxs[j]->device != ctxs[0]->device) return fail(nullptr, SL_EINVAL, "batch contexts on different devices");
        for (int k = 0; k < j; ++k)
            if (ctxs[k] == ctxs[j]) return fail(nullptr, SL_EINVAL, "context %d appears twice in the batch", j);
    }
    sl_batch* b = new sl_batch();
    b->ctxs.assign(ctxs, ctxs + n);
    b->device = ctxs[0]->device;
    if (cudaSetDevice(b->device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) ||
        cudaStreamCreateWithFlags(&b->body, cudaStreamNonBlocking) ||
        cudaEventCreateWithFlags(&b->ev_root, cudaEventDisableTiming) ||
        cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming)) {
        sl_batch_destroy(b);
        return fail(nullptr, SL_ECUDA, "creating the batch's stream");
    }
    for (int j = 0; j < n; ++j) {
        cudaStream_t st;
        cudaEvent_t ev;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) ||
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) {
            sl_batch_destroy(b);
            return fail(nullptr, SL_ECUDA, "creating the batch's streams");
        }
        b->fork.push_back(st);
        b->evs.push_back(ev);
    }
    *out = b;
    return SL_OK;
}

static int build_batch_graph(sl_batch* b) {
    b->ls_epochs.clear();
    for (sl_ctx* c : b->ctxs) {
        int rc = prepare_run_graph(c);
        if (rc) return rc;
        b->ls_epochs.push_back(c->ls_epoch);
    }
    cudaGraph_t top = nullptr;
    if (cudaGraphCreate(&top, 0) != cudaSuccess) return fail(nullptr, SL_ECUDA, "creating the batch graph");
    cudaError_t e = cudaStreamBeginCaptureToGraph(b->stream, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev_root, b->stream);
    for (size_t j = 0; j < b->ctxs.size() && e == cudaSuccess; ++j) {
        sl_ctx* c = b->ctxs[j];
        if ((e = cudaStreamWaitEvent(b->fork[j], b->ev_root, 0)) != cudaSuccess) break;
        if ((e = capture_run_nodes(c, b->fork[j], c->cap_streams[1], c->cap_streams[2])) != cudaSuccess) break;
        if ((e = cudaEventRecord(b->evs[j], b->fork[j])) != cudaSuccess) break;
        e = cudaStreamWaitEvent(b->stream, b->evs[j], 0);
    }
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &top);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, top, 0);
    cudaGraphDestroy(top);
    if (e != cudaSuccess) {
        b->graph = nullptr;
        cudaGetLastError();
        return fail(nullptr, SL_ECUDA, "capturing the batch graph: %s", cudaGetErrorString(e));
    }
    return SL_OK;
}

// A batch's MC3 run as one launch: WHILE (spurts left) { per context, in
// parallel: spurt bounds -> run nodes -> exchange -> next spurt }.  All
// contexts share the run's spurts; the first context's step decides whether
// the loop runs again.
static int build_batch_mc3_graph(sl_batch* b) {
    b->mc3_epochs.clear();
    for (sl_ctx* c : b->ctxs) {
        int rc = prepare_run_graph(c);
        if (rc) return rc;
        b->mc3_epochs.push_back(c->ls_epoch);
    }
    cudaGraph_t top = nullptr;
    if (cudaGraphCreate(&top, 0) != cudaSuccess) return fail(nullptr, SL_ECUDA, "creating the batch graph");
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaStreamBeginCaptureToGraph(b->stream, top, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        e = begin_outer_while(b->stream, b->body, &h);
        if (e == cudaSuccess) {
            e = cudaEventRecord(b->ev_root, b->body);
            for (size_t j = 0; j < b->ctxs.size() && e == cudaSuccess; ++j) {
                if ((e = cudaStreamWaitEvent(b->fork[j], b->ev_root, 0)) != cudaSuccess) break;
                if ((e = capture_mc3_spurt(b->ctxs[j], b->fork[j], h, j == 0)) != cudaSuccess) break;
                if ((e = cudaEventRecord(b->evs[j], b->fork[j])) != cudaSuccess) break;
                e = cudaStreamWaitEvent(b->body, b->evs[j], 0);
            }
            cudaGraph_t body = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(b->body, &body);
            if (e == cudaSuccess) e = e2;
        }
    }
    if ((e = end_capture(b->stream, top, e, &b->mc3_graph)) != cudaSuccess)
        return fail(nullptr, SL_ECUDA, "capturing the batch's MC3 graph: %s", cudaGetErrorString(e));
    return SL_OK;
}

int sl_batch_run(sl_batch* b, const sl_run_options* o) {
    if (!b || !o) return fail(nullptr, SL_EINVAL, "null argument");
    if (o->iterations < 0 || o->burnin < 0 || o->scoring_period < 1 || o->first_iteration < 0 ||
        o->exchange_period < 0 || !(o->lsampler_prob >= 0.0 && o->lsampler_prob <= 1.0))
        return fail(nullptr, SL_EINVAL, "bad run options");
    if (cudaSetDevice(b->device) != cudaSuccess) return fail(nullptr, SL_ECUDA, "cudaSetDevice");
    for (sl_ctx* c : b->ctxs)
        if (c->profiling) return fail(c, SL_EINVAL, "a batch runs without per-kernel profiling");
    const int total = o->burnin + o->iterations;
    const int P = o->exchange_period;
    bool paced = false;
    for (sl_ctx* c : b->ctxs) {
        ls_adopt(c);
        paced = paced || ls_compiling(c);
    }
    if (P > 0 && !paced && o->first_iteration < total) {
        // every spurt and exchange of every context in one launch
        if (b->mc3_graph)
            for (size_t j = 0; j < b->ctxs.size(); ++j)
                if (b->mc3_epochs[j] != b->ctxs[j]->ls_epoch) {
                    if (cudaStreamSynchronize(b->stream) != cudaSuccess)
                        return fail(nullptr, SL_ECUDA, "waiting for the batch graph");
                    cudaGraphExecDestroy(b->mc3_graph);
                    b->mc3_graph = nullptr;
                    break;
                }
        if (!b->mc3_graph) {
            int rc = build_batch_mc3_graph(b);
            if (rc) return rc;
        }
        for (size_t j = 0; j < b->ctxs.size(); ++j) {
            sl_ctx* c = b->ctxs[j];
            int rc = launch_mc3_run(c, o);
            if (rc) return rc;
            if (cudaEventRecord(b->evs[j], c->stream) != cudaSuccess ||
                cudaStreamWaitEvent(b->stream, b->evs[j], 0) != cudaSuccess)
                return fail(c, SL_ECUDA, "ordering the batch after the context's work");
        }
        if (cudaGraphLaunch(b->mc3_graph, b->stream) != cudaSuccess ||
            cudaEventRecord(b->ev_done, b->stream) != cudaSuccess)
            return fail(nullptr, SL_ECUDA, "launching the batch's MC3 graph");
        for (sl_ctx* c : b->ctxs)
            if (cudaStreamWaitEvent(c->stream, b->ev_done, 0) != cudaSuccess)
                return fail(c, SL_ECUDA, "ordering the context after the batch");
        return SL_OK;
    }
    for (int it0 = o->first_iteration, it1; it0 < total; it0 = it1) {
        // a context whose specialised L-sampler has compiled switches to it: the graph is captured again
        bool paced = false;
        for (sl_ctx* c : b->ctxs) {
            ls_adopt(c);
            paced = paced || ls_compiling(c);
        }
        if (b->graph)
            for (size_t j = 0; j < b->ctxs.size(); ++j)
                if (b->ls_epochs[j] != b->ctxs[j]->ls_epoch) {
                    if (cudaStreamSynchronize(b->stream) != cudaSuccess)   // no launch of it in flight
                        return fail(nullptr, SL_ECUDA, "waiting for the batch graph");
                    cudaGraphExecDestroy(b->graph);
                    b->graph = nullptr;
                    break;
                }
        if (!b->graph) {
            int rc = build_batch_graph(b);
            if (rc) return rc;
        }
        // spurts end at multiples of the exchange period counted from iteration 0 (as in sl_run);
        // while a compile runs, spans are short and waited for
        it1 = P > 0 ? std::min(total, (it0 / P + 1) * P) : total;
        if (paced) it1 = std::min(it1, it0 + kPacedSpan);
        for (size_t j = 0; j < b->ctxs.size(); ++j) {
            sl_ctx* c = b->ctxs[j];
            const RunParams rp{it0, it1, o->burnin, o->scoring_period, o->lsampler_prob, o->seed};
            if (cudaMemcpyAsync(c->d_run, &rp, sizeof(rp), cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
                cudaEventRecord(b->evs[j], c->stream) != cudaSuccess ||
                cudaStreamWaitEvent(b->stream, b->evs[j], 0) != cudaSuccess)
                return fail(c, SL_ECUDA, "ordering the batch after the context's work");
        }
        if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess || cudaEventRecord(b->ev_done, b->stream) != cudaSuccess)
            return fail(nullptr, SL_ECUDA, "launching the batch graph");
        for (sl_ctx* c : b->ctxs) {
            if (cudaStreamWaitEvent(c->stream, b->ev_done, 0) != cudaSuccess)
                return fail(c, SL_ECUDA, "ordering the context after the batch");
            account_span(c, o, it0, it1);
        }
        if (paced && cudaEventSynchronize(b->ev_done) != cudaSuccess)
            return fail(nullptr, SL_ECUDA, "waiting for a batch span");
        if (P > 0 && it1 % P == 0)
            for (sl_ctx* c : b->ctxs)
                if (c->n_chains > 1) {
                    int rc = mc3_exchange(c, o, it1);
                    if (rc) return rc;
                }
    }
    return SL_OK;
}


// ---------------------------------------------------------------------------
// Sequential imputation: legal starting graphs (SequentialImputation,
// sequential_imputation.cc:14-125; LocusSampler::start_from,
// locus_sampler2.cc:214-241).
// ---------------------------------------------------------------------------
int sl_sequential_imputation(sl_ctx* ctx, int32_t first, int32_t n_chains, const int32_t* start_loci,
                             const double* draws, int64_t chain_stride, double* weights) {
    int rc = check_chains(ctx, first, n_chains);
    if (rc) return rc;
    if (!start_loci || !draws || chain_stride < 1 || !weights) return fail(ctx, SL_EINVAL, "bad arguments");
    for (int c = 0; c < n_chains; ++c)
        if (start_loci[c] < 0 || start_loci[c] >= ctx->P.M) return fail(ctx, SL_EINVAL, "start locus out of range");
    CK(cudaSetDevice(ctx->device));
    const size_t nu = (size_t)n_chains * chain_stride;
    if (nu > ctx->u_cap) {
        if (ctx->d_u) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->d_u);
            ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), (void*)ctx->d_u));
            ctx->d_u = nullptr;
        }
        if ((rc = dev_alloc(ctx, &ctx->d_u, nu))) return rc;
        ctx->u_cap = nu;
    }
    int32_t* d_starts = nullptr;
    double* d_w = nullptr;
    if ((rc = dev_alloc(ctx, &d_starts, (size_t)n_chains))) return rc;
    if ((rc = dev_alloc(ctx, &d_w, (size_t)n_chains))) return rc;
    CK(cudaMemcpyAsync(ctx->d_u, draws, sizeof(double) * nu, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_starts, start_loci, sizeof(int32_t) * n_chains, cudaMemcpyHostToDevice, ctx->stream));
    { Prof pf_(ctx, SL_KERNEL_LSAMPLER);
    CK(launch_si(ctx->P, ctx->d_dg, first, n_chains, d_starts, ctx->d_u, chain_stride, 0, 0, d_w, ctx->d_status,
                 ctx->stream, ctx->ls_wpb, 1, 0, ctx->ls_grid)); }
    CK(cudaMemcpyAsync(weights, d_w, sizeof(double) * n_chains, cudaMemcpyDeviceToHost, ctx->stream));
    rc = sl_synchronize(ctx);
    for (void* p : {(void*)d_starts, (void*)d_w}) {
        cudaFree(p);
        ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), p));
    }
    return rc;
}

int sl_sequential_imputation_run(sl_ctx* ctx, int32_t iterations, uint64_t seed, double* best_weights) {
    if (!ctx || iterations < 1) return fail(ctx, SL_EINVAL, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    const ProblemDev& P = ctx->P;
    const int C = ctx->n_chains, M = P.M;
    const size_t words = (size_t)M * P.W;
    // passes are independent (SequentialImputation::parallel_run, sequential_imputation.cc:
    // 47-114): a batch of them runs at once, one warp per (pass, chain), its graphs in
    // scratch; the batch is bounded by a 256 MB scratch budget
    const int batch = (int)std::max<size_t>(1, std::min<size_t>((size_t)iterations,
                                                                 (256u << 20) / (sizeof(uint32_t) * words * C)));
    uint32_t* scratch = nullptr;
    int32_t* d_starts = nullptr;
    double *d_w = nullptr, *d_best = nullptr;
    int rc;
    if ((rc = dev_alloc(ctx, &scratch, words * C * batch))) return rc;
    if ((rc = dev_alloc(ctx, &d_starts, (size_t)C * batch))) return rc;
    if ((rc = dev_alloc(ctx, &d_w, (size_t)C * batch))) return rc;
    if ((rc = dev_alloc(ctx, &d_best, (size_t)C))) return rc;
    std::vector<double> lowest(C, -DBL_MAX);
    CK(cudaMemcpyAsync(d_best, lowest.data(), sizeof(double) * C, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * words * C * batch, ctx->stream));
    std::vector<int32_t> starts((size_t)C * batch);
    for (int p0 = 0; p0 < iterations; p0 += batch) {
        const int np = std::min(batch, iterations - p0);
        // each pass's start locus (get_random_locus) from its own Philox stage
        for (int q = 0; q < np; ++q)
            for (int c = 0; c < C; ++c) {
                const uint64_t hi = ((uint64_t)c << 40) ^ ((uint64_t)(p0 + q) << 4) ^ 6u;
                starts[(size_t)q * C + c] = std::min(M - 1, (int)(host_philox_u01(seed, hi, 0) * M));
            }
        CK(cudaMemcpyAsync(d_starts, starts.data(), sizeof(int32_t) * C * np, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));   // the host vector is reused next batch
        // pass q of chain c writes graph slot q * C + c of scratch
        { Prof pf_(ctx, SL_KERNEL_LSAMPLER);
        CK(launch_si(P, scratch, 0, C, d_starts, nullptr, 0, seed, (uint64_t)p0, d_w, ctx->d_status, ctx->stream,
                     ctx->ls_wpb, np, (int64_t)(words * C), ctx->ls_grid)); }
        { Prof pf_(ctx, SL_KERNEL_OTHER);
        CK(launch_si_select(scratch, ctx->d_dg, 0, C, words, d_w, d_best, np, ctx->stream)); }
    }
    if (best_weights)
        CK(cudaMemcpyAsync(best_weights, d_best, sizeof(double) * C, cudaMemcpyDeviceToHost, ctx->stream));
    rc = sl_synchronize(ctx);
    for (void* p : {(void*)scratch, (void*)d_starts, (void*)d_w, (void*)d_best}) {
        cudaFree(p);
        ctx->owned.erase(std::find(ctx->owned.begin(), ctx->owned.end(), p));
    }
    if (!rc && best_weights)
        for (int c = 0; c < C; ++c)
            if (best_weights[c] == -DBL_MAX)
                return fail(ctx, SL_EZERO, "sequential imputation produced no legal graph for chain %d", c);
    return rc;
}

int sl_mc3_stats(sl_ctx* ctx, int64_t* accepted, int64_t* proposed) {
    if (!ctx) return fail(ctx, SL_EINVAL, "null context");
    CK(cudaSetDevice(ctx->device));
    const size_t n = ctx->swap_accept.size();
    CK(cudaMemcpyAsync(ctx->swap_accept.data(), ctx->d_swap_acc, sizeof(int64_t) * n, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaMemcpyAsync(ctx->swap_propose.data(), ctx->d_swap_prop, sizeof(int64_t) * n, cudaMemcpyDeviceToHost,
                       ctx->stream));
    int rc = sl_synchronize(ctx);
    if (rc) return rc;
    for (int c = 0; c + 1 < ctx->n_chains; ++c) {
        if (accepted) accepted[c] = ctx->swap_accept[c];
        if (proposed) proposed[c] = ctx->swap_propose[c];
    }
    return SL_OK;
}

int sl_chain_loglik(sl_ctx* ctx, int32_t graph_chain, int32_t map_chain, double* loglik) {
    if (!ctx || !loglik) return fail(ctx, SL_EINVAL, "null argument");
    if (graph_chain < 0 || graph_chain >= ctx->n_chains || map_chain < 0 || map_chain >= ctx->n_chains)
        return fail(ctx, SL_EINVAL, "chain outside [0, %d)", ctx->n_chains);
    CK(cudaSetDevice(ctx->device));
    return loglik_pairs(ctx, &graph_chain, &map_chain, 1, loglik);
}

}  // extern "C"
