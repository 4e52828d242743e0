/* TEST INFRASTRUCTURE ONLY: plain-C restatement of the reference's CPU hot
 * path (L-sampler, M-sampler, trait-peel LOD scorer).  It is the checker the
 * CUDA kernels are compared with and the CPU port timed by bench.py's
 * cpu_baseline leg; the product never calls it.  Each function names the
 * reference file:line it follows.  The order of every floating-point
 * operation matches the reference so that the sampler decisions are
 * bit-identical; the build uses -ffp-contract=off for the same reason.
 */
#include "sl_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { UU = 0, AA = 1, AU = 2, UA = 3 };                  /* trait.h:21-27 */
enum { G_UNTYPED = 0, G_HETERO = 1, G_HOMOZ_A = 2, G_HOMOZ_B = 3 }; /* genotype.h:26-31 */
enum { T_U = 0, T_A = 1 };
enum { CHILD = 1, PARENT = 2, PARTNER = 3, LAST = 4 };    /* peeling.h:16-22 */

static inline int dgget(const slo_problem* p, const int32_t* dg, int person, int locus, int parent) {
    return dg[(size_t)2 * p->N * locus + 2 * person + parent];
}

static inline void dgset(const slo_problem* p, int32_t* dg, int person, int locus, int parent, int v) {
    dg[(size_t)2 * p->N * locus + 2 * person + parent] = v;
}

static inline int ipow4(int c) { return 1 << (2 * c); }

/* ---------------------------------------------------------------------------
 * L-sampler (sampler_rfunction.cc, rfunction.cc, locus_sampler2.cc)
 * ------------------------------------------------------------------------- */

/* get_recombination_distribution (sampler_rfunction.cc:102-157) */
/* has_left / has_right: the neighbouring loci the step may use; false at the
   ends of the map and where sequential imputation ignores a side
   (set_locus(l, ignore_left, ignore_right), sampler_rfunction.h:84-101) */
static int g_has_left = -1, g_has_right = -1;   /* -1: decided by the locus */

static int use_left(const slo_problem* p, int locus) { return g_has_left < 0 ? locus != 0 : g_has_left; }
static int use_right(const slo_problem* p, int locus) { return g_has_right < 0 ? locus != p->M - 1 : g_has_right; }

static void recomb_dist(const slo_problem* p, const int32_t* dg, int locus, int person, int parent_trait,
                        int parent, double* dist) {
    if (parent_trait == UU) { dist[T_U] = 1.0; dist[T_A] = 0.0; return; }
    if (parent_trait == AA) { dist[T_U] = 0.0; dist[T_A] = 1.0; return; }
    double tmp0 = 0.5, tmp1 = 0.5;
    if (use_left(p, locus)) {
        int cross = dgget(p, dg, person, locus - 1, parent) != 0;
        double th2 = p->theta[locus - 1], an2 = 1.0 - p->theta[locus - 1];
        tmp0 *= (cross ? th2 : an2);
        tmp1 *= (cross ? an2 : th2);
    }
    if (use_right(p, locus)) {
        int cross = dgget(p, dg, person, locus + 1, parent) != 0;
        double th = p->theta[locus], an = 1.0 - p->theta[locus];
        tmp0 *= (cross ? th : an);
        tmp1 *= (cross ? an : th);
    }
    double total = tmp0 + tmp1;
    if (parent_trait == AU) {
        dist[T_U] = tmp1 / total;
        dist[T_A] = 1.0 - dist[T_U];
    } else {
        dist[T_U] = tmp0 / total;
        dist[T_A] = 1.0 - dist[T_U];
    }
}

/* transmission_matrix (sampler_rfunction.cc:350-419): T[m*16 + p*4 + k] */
static void transmission(const slo_problem* p, const int32_t* dg, int locus, int kid, double* T) {
    double md[2], pd[2];
    for (int i = 0; i < 4; ++i) {
        recomb_dist(p, dg, locus, kid, i, 0, md);
        for (int j = 0; j < 4; ++j) {
            int b = 16 * i + 4 * j;
            recomb_dist(p, dg, locus, kid, j, 1, pd);
            T[b + UU] = md[T_U] * pd[T_U];
            T[b + AU] = md[T_A] * pd[T_U];
            T[b + UA] = md[T_U] * pd[T_A];
            T[b + AA] = md[T_A] * pd[T_A];
        }
    }
}

typedef struct {
    double** mat;     /* [K][4^c] */
    double** pre;     /* [K][4^(c+1)] */
    double* T;        /* [N][64] transmission per child, filled on demand */
    int* assign;      /* [N] */
} lws;

static int cut_len(const slo_problem* p, int k) { return p->cut_off[k + 1] - p->cut_off[k]; }

/* index of a prev rfunction's matrix cell (peel_matrix.h:37-45) */
static inline int prev_index(const slo_problem* p, int j, const int* assign) {
    int idx = 0;
    for (int q = p->cut_off[j]; q < p->cut_off[j + 1]; ++q)
        idx += assign[p->cut[q]] << (2 * (q - p->cut_off[j]));
    return idx;
}

static double g_last_root = 0.0;

/* Decision margins: the smallest |draw - boundary| of the sampling decisions
 * since slo_margin_reset (the cumulative sums a draw is compared with in
 * SamplerRfunction::sample, the homozygous-parent indicator threshold, the
 * M-sampler's backward threshold).  A draw this close to a boundary can go
 * either way under another rounding; the fast (FP32) samplers are checked
 * against it.  Test instrumentation only: it changes no decision. */
static double g_margin = 1.0;
static inline void note_margin(double r, double b) {
    double m = fabs(r - b);
    if (m < g_margin) g_margin = m;
}
void slo_margin_reset(void) { g_margin = 1.0; }
double slo_margin(void) { return g_margin; }
/* per-locus margins of the M-step's backward draws (1 where no draw was taken) */
static double* g_mlog = NULL;
void slo_margin_log(double* per_locus) { g_mlog = per_locus; }

static void lws_alloc(const slo_problem* p, lws* w) {
    int N = p->N, K = p->K;
    w->mat = (double**)calloc(K, sizeof(double*));
    w->pre = (double**)calloc(K, sizeof(double*));
    w->T = (double*)calloc((size_t)N * 64, sizeof(double));
    w->assign = (int*)malloc(sizeof(int) * N);
    for (int k = 0; k < K; ++k) {
        int c = cut_len(p, k);
        w->mat[k] = (double*)calloc(ipow4(c), sizeof(double));
        w->pre[k] = (double*)calloc(ipow4(c + 1), sizeof(double));
    }
}

static void lws_free(const slo_problem* p, lws* w) {
    for (int k = 0; k < p->K; ++k) { free(w->mat[k]); free(w->pre[k]); }
    free(w->mat); free(w->pre); free(w->T); free(w->assign);
}

/* one L-step on a workspace whose matrices are zero (cells the step does not
   write -- invalid cells, zero-prior states -- read as 0, as in a fresh
   PeelMatrix); the step leaves them zero again for the next call */
static int lstep_ws(const slo_problem* p, lws* wp, int32_t* dg, int locus, const double* u, int n_u, int* n_used);

int slo_lstep(const slo_problem* p, int32_t* dg, int locus, const double* u, int n_u, int* n_used) {
    lws w;
    lws_alloc(p, &w);
    int rc = lstep_ws(p, &w, dg, locus, u, n_u, n_used);
    lws_free(p, &w);
    return rc;
}

/* L-steps at the listed loci, in list order, in place, with one workspace;
 * loci[i]'s draws start at u[i * u_stride]. */
int slo_lsteps(const slo_problem* p, int32_t* dg, const int32_t* loci, int n, const double* u, int u_stride) {
    lws w;
    lws_alloc(p, &w);
    int rc = 0;
    for (int i = 0; i < n && !rc; ++i) {
        int used = 0;
        rc = lstep_ws(p, &w, dg, loci[i], u + (size_t)i * u_stride, u_stride, &used);
    }
    lws_free(p, &w);
    return rc;
}

/* A full L-sweep (the device's schedule: every even locus, then every odd
 * locus, each set non-interfering, markov_chain.cc:406-416) in one call with
 * one workspace; locus l's draws start at u[l * u_stride]. */
int slo_lsweep(const slo_problem* p, int32_t* dg, const double* u, int u_stride) {
    lws w;
    lws_alloc(p, &w);
    int rc = 0;
    for (int par = 0; par < 2 && !rc; ++par)
        for (int l = par; l < p->M && !rc; l += 2) {
            int n = 0;
            rc = lstep_ws(p, &w, dg, l, u + (size_t)l * u_stride, u_stride, &n);
        }
    lws_free(p, &w);
    return rc;
}

static int lstep_ws(const slo_problem* p, lws* wp, int32_t* dg, int locus, const double* u, int n_u, int* n_used) {
    int N = p->N, K = p->K;
    lws w = *wp;
    int used = 0, rc = 0;
    /* forward peel (rfunction.cc:172-198 with offset 0) */
    for (int k = 0; k < K; ++k) {
        int c = cut_len(p, k);
        const int* cs = p->cut + p->cut_off[k];
        int peel = p->op_peel[k];
        int type = p->op_type[k];
        const double* trait = p->prior + ((size_t)locus * N + peel) * 4;
        /* populate_transmission_cache (sampler_rfunction.cc:327-341) */
        if (type == CHILD) transmission(p, dg, locus, peel, w.T + (size_t)peel * 64);
        if (type == PARENT)
            for (int q = p->ch_off[k]; q < p->ch_off[k + 1]; ++q)
                transmission(p, dg, locus, p->ch[q], w.T + (size_t)p->ch[q] * 64);
        int ncell = ipow4(c);
        for (int cell = 0; cell < ncell; ++cell) {
            int valid = 1;
            for (int q = 0; q < c; ++q) {
                int v = (cell >> (2 * q)) & 3;
                w.assign[cs[q]] = v;
                if (!((p->legal[(size_t)locus * N + cs[q]] >> v) & 1)) valid = 0;
            }
            if (!valid) continue;  /* matrix_indices (peel_sequence_generator.cc:131-150) */
            double total = 0.0;
            if (type == CHILD) {  /* sampler_rfunction.cc:190-233 */
                int mt = w.assign[p->mother[peel]], pt = w.assign[p->father[peel]];
                for (int i = 0; i < 4; ++i) {
                    w.assign[peel] = i;
                    double tmp = trait[i];
                    if (tmp == 0.0) continue;
                    tmp *= w.T[(size_t)peel * 64 + mt * 16 + pt * 4 + i];
                    for (int q = p->prev_off[k]; q < p->prev_off[k + 1]; ++q) {
                        int j = p->prev[q];
                        tmp *= w.mat[j][prev_index(p, j, w.assign)];
                    }
                    w.pre[k][cell + ncell * i] = tmp;
                    total += tmp;
                }
            } else if (type == PARENT) {  /* sampler_rfunction.cc:236-287 */
                for (int i = 0; i < 4; ++i) {
                    int mt = i, pt = i;
                    w.assign[peel] = i;
                    double tmp = trait[i];
                    if (tmp == 0.0) continue;
                    for (int q = p->prev_off[k]; q < p->prev_off[k + 1]; ++q) {
                        int j = p->prev[q];
                        tmp *= w.mat[j][prev_index(p, j, w.assign)];
                    }
                    double child_prob = 1.0;
                    for (int q = p->ch_off[k]; q < p->ch_off[k + 1]; ++q) {
                        int ch = p->ch[q];
                        int kt = w.assign[ch];
                        if (p->mother[ch] == peel) pt = w.assign[p->father[ch]];
                        else mt = w.assign[p->mother[ch]];
                        child_prob *= w.T[(size_t)ch * 64 + mt * 16 + pt * 4 + kt];
                    }
                    tmp *= child_prob;
                    w.pre[k][cell + ncell * i] = tmp;
                    total += tmp;
                }
            } else {  /* partner / last: rfunction.cc:116-142 */
                for (int i = 0; i < 4; ++i) {
                    w.assign[peel] = i;
                    double tmp = trait[i];
                    if (tmp == 0.0) continue;
                    for (int q = p->prev_off[k]; q < p->prev_off[k + 1]; ++q) {
                        int j = p->prev[q];
                        tmp *= w.mat[j][prev_index(p, j, w.assign)];
                    }
                    w.pre[k][cell + ncell * i] = tmp;
                    total += tmp;
                }
            }
            w.mat[k][cell] = total;
        }
    }
    if (w.mat[K - 1][0] == 0.0) { rc = -1; goto done; }  /* locus_sampler2.cc:137-142 */
    g_last_root = w.mat[K - 1][0];
    /* backward sampling (locus_sampler2.cc:146-148, sampler_rfunction.cc:159-188) */
    for (int i = 0; i < N; ++i) w.assign[i] = -1;
    for (int k = K - 1; k >= 0; --k) {
        int c = cut_len(p, k);
        const int* cs = p->cut + p->cut_off[k];
        int peel = p->op_peel[k];
        int base = 0;
        for (int q = 0; q < c; ++q) base += w.assign[cs[q]] << (2 * q);
        double pd[4];
        for (int v = 0; v < 4; ++v) pd[v] = w.pre[k][base + ipow4(c) * v];
        double tot = pd[0] + pd[1] + pd[2] + pd[3];
        if (tot != 0.0)
            for (int v = 0; v < 4; ++v) pd[v] /= tot;
        if (used >= n_u) { rc = -2; goto done; }
        double r = u[used++];
        double acc = 0.0;
        int last = 0, pick = -1;
        {
            double a2 = 0.0;   /* every boundary the draw could fall on */
            for (int v = 0; v < 3; ++v) { a2 += pd[v]; if (pd[v] != 0.0) note_margin(r, a2); }
        }
        for (int v = 0; v < 4; ++v) {
            acc += pd[v];
            if (r < acc) { pick = v; break; }
            if (pd[v] != 0.0) last = v;
        }
        w.assign[peel] = pick >= 0 ? pick : last;
    }
    /* sample_meiosis_indicators (locus_sampler2.cc:93-125) */
    for (int i = 0; i < N; ++i) {
        if (p->mother[i] < 0) continue;
        int tr = w.assign[i];
        for (int par = 0; par < 2; ++par) {
            int ptr = w.assign[par == 0 ? p->mother[i] : p->father[i]];
            int allele = (par == 0) ? ((tr == UU || tr == UA) ? T_U : T_A)
                                    : ((tr == UU || tr == AU) ? T_U : T_A);
            int mi;
            if (ptr == UA || ptr == AU) {  /* sample_hetero_mi (locus_sampler2.cc:32-42) */
                if (allele == T_U) mi = (ptr == UA) ? 0 : 1;
                else mi = (ptr == UA) ? 1 : 0;
            } else {  /* sample_homo_mi (locus_sampler2.cc:44-65) */
                double p0 = 1.0, p1 = 1.0;
                if (use_left(p, locus)) {
                    int d = dgget(p, dg, i, locus - 1, par);
                    double th = p->theta[locus - 1], an = 1.0 - p->theta[locus - 1];
                    p0 *= (d == 0) ? an : th;
                    p1 *= (d == 1) ? an : th;
                }
                if (use_right(p, locus)) {
                    int d = dgget(p, dg, i, locus + 1, par);
                    double th = p->theta[locus], an = 1.0 - p->theta[locus];
                    p0 *= (d == 0) ? an : th;
                    p1 *= (d == 1) ? an : th;
                }
                if (used >= n_u) { rc = -2; goto done; }
                note_margin(u[used], p0 / (p0 + p1));
                mi = (u[used++] < (p0 / (p0 + p1))) ? 0 : 1;
            }
            dgset(p, dg, i, locus, par, mi);
        }
    }
done:
    *n_used = used;
    for (int k = 0; k < K; ++k) {
        int c = cut_len(p, k);
        memset(w.mat[k], 0, sizeof(double) * ipow4(c));
        memset(w.pre[k], 0, sizeof(double) * ipow4(c + 1));
    }
    return rc;
}

/* ---------------------------------------------------------------------------
 * Founder allele graph (founder_allele_graph4.cc:34-442)
 * ------------------------------------------------------------------------- */

typedef struct {
    int* edge;       /* [2N] founder allele of each person's maternal/paternal allele */
    int* order;      /* [N] topological order, founders first */
    int* member;     /* [2F] */
    int* fixed;      /* [2F] */
    unsigned char* active;
    int* a0;         /* allele_assignment[0][fa] */
    int* a1;
    double* pr0;     /* prob[0][group] */
    double* pr1;
} fws;

static void fws_init(const slo_problem* p, fws* f) {
    int N = p->N, nfa = 2 * p->F;
    f->edge = (int*)malloc(sizeof(int) * 2 * N);
    f->order = (int*)malloc(sizeof(int) * N);
    f->member = (int*)malloc(sizeof(int) * nfa);
    f->fixed = (int*)malloc(sizeof(int) * nfa);
    f->active = (unsigned char*)malloc(nfa);
    f->a0 = (int*)malloc(sizeof(int) * nfa);
    f->a1 = (int*)malloc(sizeof(int) * nfa);
    f->pr0 = (double*)malloc(sizeof(double) * nfa);
    f->pr1 = (double*)malloc(sizeof(double) * nfa);
    /* find_founderallelegraph_ordering (descent_graph.cc:320-355) */
    unsigned char* vis = (unsigned char*)calloc(N, 1);
    int n = 0;
    for (int i = 0; i < p->F; ++i) { f->order[n++] = i; vis[i] = 1; }
    while (n < N) {
        for (int i = p->F; i < N; ++i) {
            if (vis[i]) continue;
            if (vis[p->mother[i]] && vis[p->father[i]]) { f->order[n++] = i; vis[i] = 1; }
        }
    }
    free(vis);
}

static void fws_free(fws* f) {
    free(f->edge); free(f->order); free(f->member); free(f->fixed); free(f->active);
    free(f->a0); free(f->a1); free(f->pr0); free(f->pr1);
}

/* FounderAlleleGraph4::reset (founder_allele_graph4.cc:543-569); the
 * optional flip toggles one meiosis, which equals flip() + propagation
 * (founder_allele_graph4.cc:571-597) applied to the same column. */
static void fag_edges(const slo_problem* p, const int32_t* dg, int locus, fws* f, int flip_person,
                      int flip_parent) {
    for (int n = 0; n < p->N; ++n) {
        int pid = f->order[n];
        if (p->mother[pid] < 0) {
            f->edge[2 * pid] = 2 * pid;
            f->edge[2 * pid + 1] = 2 * pid + 1;
        } else {
            int vm = dgget(p, dg, pid, locus, 0), vp = dgget(p, dg, pid, locus, 1);
            if (pid == flip_person) {
                if (flip_parent == 0) vm ^= 1; else vp ^= 1;
            }
            f->edge[2 * pid] = f->edge[2 * p->mother[pid] + vm];
            f->edge[2 * pid + 1] = f->edge[2 * p->father[pid] + vp];
        }
    }
}

static inline int fag_legal(int obs, int x, int y) {
    switch (obs) {
        case G_HETERO: return x != y;
        case G_HOMOZ_A: return x == G_HOMOZ_A && y == G_HOMOZ_A;
        case G_HOMOZ_B: return x == G_HOMOZ_B && y == G_HOMOZ_B;
    }
    return 0;
}

static inline int fag_other(int obs, int x) {
    switch (obs) {
        case G_HETERO: return x == G_HOMOZ_A ? G_HOMOZ_B : G_HOMOZ_A;
        case G_HOMOZ_A: return x == G_HOMOZ_A ? G_HOMOZ_A : G_UNTYPED;
        case G_HOMOZ_B: return x == G_HOMOZ_B ? G_HOMOZ_B : G_UNTYPED;
    }
    return G_UNTYPED;
}

static void fag_combine(fws* f, int nfa, int c1, int c2, int flip) {
    for (int i = 0; i < nfa; ++i) {
        if (f->member[i] == c2) {
            f->member[i] = c1;
            if (flip) { int t = f->a0[i]; f->a0[i] = f->a1[i]; f->a1[i] = t; }
        }
    }
    if (flip) {
        f->pr0[c1] *= f->pr1[c2];
        f->pr1[c1] *= f->pr0[c2];
    } else {
        f->pr0[c1] *= f->pr0[c2];
        f->pr1[c1] *= f->pr1[c2];
    }
    f->active[c2] = 0;
}

#define ASG(f, w, fa) ((w) == 0 ? (f)->a0[fa] : (f)->a1[fa])
#define PRB(f, w, g) (*((w) == 0 ? &(f)->pr0[g] : &(f)->pr1[g]))

static double fag_like(const slo_problem* p, int locus, fws* f) {
    int nfa = 2 * p->F;
    double minor = p->minor[locus], major = 1.0 - p->minor[locus];
    for (int i = 0; i < nfa; ++i) {
        f->member[i] = -1; f->fixed[i] = -1; f->active[i] = 0; f->a0[i] = 0; f->a1[i] = 0;
    }
    int gi = 0;
#define FREQ(g) ((g) == G_HOMOZ_A ? major : minor)
    for (int i = 0; i < p->N; ++i) {
        if (!p->typed[i]) continue;
        int g = p->geno[(size_t)locus * p->N + i];
        if (g == G_UNTYPED) continue;
        int mfa = f->edge[2 * i], pfa = f->edge[2 * i + 1];
        if (mfa == pfa) {
            if (g == G_HETERO) return 0.0;
            int g1 = f->member[mfa];
            if (g1 != -1) {
                int f1 = f->fixed[g1];
                if (f1 != -1) {
                    if (g != ASG(f, f1, mfa)) return 0.0;
                } else {
                    if (f->a0[mfa] == g) { f->fixed[g1] = 0; f->pr1[g1] = 0.0; }
                    else if (f->a1[mfa] == g) { f->fixed[g1] = 1; f->pr0[g1] = 0.0; }
                    else return 0.0;
                }
            } else {
                f->member[mfa] = gi; f->fixed[gi] = 0; f->active[gi] = 1;
                f->a0[mfa] = g; f->pr0[gi] = FREQ(g); f->pr1[gi] = 0.0;
                ++gi;
            }
            continue;
        }
        int g1 = f->member[mfa], g2 = f->member[pfa];
        if (g1 != -1) {
            int f1 = f->fixed[g1];
            if (g2 != -1) {
                if (g1 == g2) {
                    if (f1 != -1) {
                        if (!fag_legal(g, ASG(f, f1, mfa), ASG(f, f1, pfa))) return 0.0;
                    } else {
                        int l0 = fag_legal(g, f->a0[mfa], f->a0[pfa]);
                        int l1 = fag_legal(g, f->a1[mfa], f->a1[pfa]);
                        if (l0) {
                            if (!l1) { f->fixed[g1] = 0; f->pr1[g1] = 0.0; }
                        } else {
                            if (l1) { f->fixed[g1] = 1; f->pr0[g1] = 0.0; }
                            else return 0.0;
                        }
                    }
                } else {
                    int f2 = f->fixed[g2];
                    if (f1 != -1) {
                        if (f2 != -1) {
                            if (!fag_legal(g, ASG(f, f1, mfa), ASG(f, f2, pfa))) return 0.0;
                        } else {
                            int l0 = fag_legal(g, ASG(f, f1, mfa), f->a0[pfa]);
                            int l1 = fag_legal(g, ASG(f, f1, mfa), f->a1[pfa]);
                            if (l0) f2 = 0; else if (l1) f2 = 1; else return 0.0;
                        }
                    } else if (f2 != -1) {
                        int l0 = fag_legal(g, f->a0[mfa], ASG(f, f2, pfa));
                        int l1 = fag_legal(g, f->a1[mfa], ASG(f, f2, pfa));
                        if (l0) f1 = 0; else if (l1) f1 = 1; else return 0.0;
                    } else {
                        int l0 = fag_legal(g, f->a0[mfa], f->a0[pfa]);
                        int l1 = fag_legal(g, f->a1[mfa], f->a0[pfa]);
                        int l2 = fag_legal(g, f->a0[mfa], f->a1[pfa]);
                        int l3 = fag_legal(g, f->a1[mfa], f->a1[pfa]);
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
                        f->fixed[g1] = f1;
                        PRB(f, 1 - f1, g1) = 0.0;
                        PRB(f, 1 - f2, g2) = 0.0;
                        fag_combine(f, nfa, g1, g2, 1);
                    } else if (f1 == -2) {
                        f->fixed[g1] = -1;
                        fag_combine(f, nfa, g1, g2, 1);
                    } else {
                        f->fixed[g1] = f1;
                        if (f1 != -1) {
                            PRB(f, 1 - f1, g1) = 0.0;
                            PRB(f, 1 - f2, g2) = 0.0;
                        }
                        fag_combine(f, nfa, g1, g2, 0);
                    }
                }
            } else {
                if (f1 != -1) {
                    int t0 = fag_other(g, ASG(f, f1, mfa));
                    if (t0 == G_UNTYPED) return 0.0;
                    if (f1 == 0) f->a0[pfa] = t0; else f->a1[pfa] = t0;
                    PRB(f, f1, g1) *= FREQ(t0);
                } else {
                    int t0 = fag_other(g, f->a0[mfa]);
                    int t1 = fag_other(g, f->a1[mfa]);
                    if (t0 != G_UNTYPED) {
                        if (t1 != G_UNTYPED) {
                            f->a0[pfa] = t0; f->a1[pfa] = t1;
                            f->pr0[g1] *= FREQ(t0);
                            f->pr1[g1] *= FREQ(t1);
                        } else {
                            f->a0[pfa] = t0;
                            f->pr0[g1] *= FREQ(t0);
                            f->pr1[g1] = 0.0;
                            f->fixed[g1] = 0;
                        }
                    } else {
                        if (t1 != G_UNTYPED) {
                            f->a1[pfa] = t1;
                            f->pr1[g1] *= FREQ(t1);
                            f->pr0[g1] = 0.0;
                            f->fixed[g1] = 1;
                        } else return 0.0;
                    }
                }
                f->member[pfa] = g1;
            }
        } else if (g2 != -1) {
            int f2 = f->fixed[g2];
            if (f2 != -1) {
                int t0 = fag_other(g, ASG(f, f2, pfa));
                if (t0 == G_UNTYPED) return 0.0;
                if (f2 == 0) f->a0[mfa] = t0; else f->a1[mfa] = t0;
                PRB(f, f2, g2) *= FREQ(t0);
            } else {
                int t0 = fag_other(g, f->a0[pfa]);
                int t1 = fag_other(g, f->a1[pfa]);
                if (t0 != G_UNTYPED) {
                    if (t1 != G_UNTYPED) {
                        f->a0[mfa] = t0; f->a1[mfa] = t1;
                        f->pr0[g2] *= FREQ(t0);
                        f->pr1[g2] *= FREQ(t1);
                    } else {
                        f->a0[mfa] = t0;
                        f->pr0[g2] *= FREQ(t0);
                        f->pr1[g2] = 0.0;
                        f->fixed[g2] = 0;
                    }
                } else {
                    if (t1 != G_UNTYPED) {
                        f->a1[mfa] = t1;
                        f->pr1[g2] *= FREQ(t1);
                        f->pr0[g2] = 0.0;
                        f->fixed[g2] = 1;
                    } else return 0.0;
                }
            }
            f->member[mfa] = g2;
        } else {
            if (g == G_HETERO) {
                f->a0[mfa] = G_HOMOZ_A; f->a1[pfa] = G_HOMOZ_A;
                f->a1[mfa] = G_HOMOZ_B; f->a0[pfa] = G_HOMOZ_B;
                f->pr0[gi] = major * minor;
                f->pr1[gi] = major * minor;
                f->fixed[gi] = -1;
            } else {
                f->a0[mfa] = g; f->a0[pfa] = g;
                f->pr0[gi] = FREQ(g) * FREQ(g);
                f->pr1[gi] = 0.0;
                f->fixed[gi] = 0;
            }
            f->member[mfa] = gi; f->member[pfa] = gi;
            f->active[gi] = 1;
            ++gi;
        }
    }
#undef FREQ
    double ret = 1.0;
    for (int i = 0; i < gi; ++i) {
        if (!f->active[i]) continue;
        int fx = f->fixed[i];
        if (fx != -1) ret *= PRB(f, fx, i);
        else ret *= (f->pr0[i] + f->pr1[i]);
    }
    return ret;
}

double slo_fag_likelihood(const slo_problem* p, const int32_t* dg, int locus) {
    fws f;
    fws_init(p, &f);
    fag_edges(p, dg, locus, &f, -1, 0);
    double r = fag_like(p, locus, &f);
    fws_free(&f);
    return r;
}

/* ---------------------------------------------------------------------------
 * M-sampler (meiosis_sampler.cc:17-203)
 * ------------------------------------------------------------------------- */

int slo_msweep(const slo_problem* p, int32_t* dg, const int32_t* meioses, int n, const double* u,
               int32_t* n_used) {
    int M = p->M, F = p->F;
    double* raw = (double*)malloc(sizeof(double) * 2 * M);
    double* fb = (double*)malloc(sizeof(double) * 2 * M);
    fws f;
    fws_init(p, &f);
    int rc = 0;
    /* reset (meiosis_sampler.cc:17-40) */
    int m0 = meioses[0];
    int person = F + m0 / 2, par = m0 % 2;
    for (int l = 0; l < M; ++l) {
        fag_edges(p, dg, l, &f, -1, 0);
        int cur = dgget(p, dg, person, l, par);
        raw[2 * l + cur] = fag_like(p, l, &f);
        if (raw[2 * l + cur] == 0.0) { rc = -1; goto out; }
    }
    int last = m0;
    for (int s = 0; s < n; ++s) {
        int m = meioses[s];
        person = F + m / 2; par = m % 2;
        int lperson = F + last / 2, lpar = last % 2;
        const double* us = u + (size_t)s * M;
        int used = 0;
        /* meiosis_sampler.cc:116-133 */
        for (int l = 0; l < M; ++l) {
            int t = dgget(p, dg, person, l, par);
            int t2 = dgget(p, dg, lperson, l, lpar);
            raw[2 * l + t] = raw[2 * l + t2];
            fag_edges(p, dg, l, &f, person, par);
            raw[2 * l + (1 - t)] = fag_like(p, l, &f);
            if (raw[2 * l] == 0.0 && raw[2 * l + 1] == 0.0) { rc = -1; goto out; }
        }
        /* forward filter (meiosis_sampler.cc:136-155) */
        double total = raw[0] + raw[1];
        fb[0] = raw[0] / total;
        fb[1] = raw[1] / total;
        for (int i = 1; i < M; ++i) {
            double th = p->theta[i - 1], an = 1.0 - p->theta[i - 1];
            for (int j = 0; j < 2; ++j)
                fb[2 * i + j] = raw[2 * i + j] * ((fb[2 * (i - 1) + (1 - j)] * th) + (fb[2 * (i - 1) + j] * an));
            double tt = fb[2 * i] + fb[2 * i + 1];
            fb[2 * i] /= tt;
            fb[2 * i + 1] /= tt;
        }
        /* backward sampling (meiosis_sampler.cc:157-203) */
        for (int i = M - 1; i >= 0; --i) {
            if (i < M - 1) {
                int nxt = dgget(p, dg, person, i + 1, par);
                double th = p->theta[i], an = 1.0 - p->theta[i];
                for (int j = 0; j < 2; ++j) fb[2 * i + j] *= (nxt != j) ? th : an;
            }
            int samp;
            if (g_mlog) g_mlog[i] = 1.0;
            if (fb[2 * i] == 0.0) samp = 1;
            else if (fb[2 * i + 1] == 0.0) samp = 0;
            else {
                note_margin(us[used], fb[2 * i] / (fb[2 * i] + fb[2 * i + 1]));
                if (g_mlog) g_mlog[i] = fabs(us[used] - fb[2 * i] / (fb[2 * i] + fb[2 * i + 1]));
                samp = (us[used++] < (fb[2 * i] / (fb[2 * i] + fb[2 * i + 1]))) ? 0 : 1;
            }
            if (samp != dgget(p, dg, person, i, par)) dgset(p, dg, person, i, par, samp);
        }
        n_used[s] = used;
        last = m;
    }
out:
    fws_free(&f);
    free(raw);
    free(fb);
    return rc;
}

/* ---------------------------------------------------------------------------
 * Trait peel and LOD scores (trait_rfunction.cc, peeler.cc, lod_score.h)
 * ------------------------------------------------------------------------- */

static inline int affected_trait(int pt, int allele) {  /* rfunction.h:82-107 */
    switch (pt) {
        case UU: return 0;
        case AU: return allele == 0;
        case UA: return allele == 1;
        case AA: return 1;
    }
    return 0;
}

static inline int phased_trait(int m, int pt, int i, int j) {  /* rfunction.cc:98-114 */
    int ma = affected_trait(m, i), pa = affected_trait(pt, j);
    if (ma) return pa ? AA : AU;
    return pa ? UA : UU;
}

typedef struct {
    const int32_t* dg;
    int locus;
    double th, an, th2, an2;
} tctx;

/* TraitRfunction::get_recombination_probability (trait_rfunction.cc:9-24) */
static inline double trait_rec(const slo_problem* p, const tctx* t, int person, int i, int j) {
    double tmp = 1.0;
    tmp *= (dgget(p, t->dg, person, t->locus, 0) == i) ? t->an : t->th;
    tmp *= (dgget(p, t->dg, person, t->locus + 1, 0) == i) ? t->an2 : t->th2;
    tmp *= (dgget(p, t->dg, person, t->locus, 1) == j) ? t->an : t->th;
    tmp *= (dgget(p, t->dg, person, t->locus + 1, 1) == j) ? t->an2 : t->th2;
    return tmp;
}

/* one full trait peel; returns the final rfunction value (peeler.cc:79-91).
 * esum NULL: the reference's plain FP64 peel.  esum non-NULL: after each
 * rfunction is complete, its cells are divided by 2^e, e the binary exponent
 * of its largest valid cell (frexp), and e is added to *esum; the peel's value
 * is then the returned value times 2^(*esum).  Dividing by a power of two is
 * exact, so away from underflow the two forms agree to the last rounding of
 * the logarithm, and the rescaled form does not underflow where the plain one
 * does (hundreds of members). */
static double trait_peel(const slo_problem* p, const tctx* t, double** mat, int* assign, long* esum) {
    int N = p->N;
    if (esum) *esum = 0;
    for (int k = 0; k < p->K; ++k) {
        double vmax = 0.0;
        int c = cut_len(p, k);
        const int* cs = p->cut + p->cut_off[k];
        int peel = p->op_peel[k], type = p->op_type[k];
        const double* trait = p->dprob + (size_t)peel * 4;
        int ncell = ipow4(c);
        for (int cell = 0; cell < ncell; ++cell) {
            int valid = 1;
            for (int q = 0; q < c; ++q) {
                int v = (cell >> (2 * q)) & 3;
                assign[cs[q]] = v;
                if (p->dprob[(size_t)cs[q] * 4 + v] == 0.0) valid = 0;
            }
            if (!valid) continue;  /* lod_indices (peel_sequence_generator.cc:155-179) */
            double total = 0.0;
            if (type == CHILD) {  /* trait_rfunction.cc:30-69 */
                int mt = assign[p->mother[peel]], pt = assign[p->father[peel]];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) {
                        int kt = phased_trait(mt, pt, i, j);
                        assign[peel] = kt;
                        double tmp = trait[kt];
                        if (tmp == 0.0) continue;
                        for (int q = p->prev_off[k]; q < p->prev_off[k + 1]; ++q) {
                            int jj = p->prev[q];
                            tmp *= mat[jj][prev_index(p, jj, assign)];
                        }
                        tmp *= (t->dg == NULL) ? 0.25 : 0.25 * trait_rec(p, t, peel, i, j);
                        total += tmp;
                    }
            } else if (type == PARENT) {  /* trait_rfunction.cc:71-137 */
                for (int a = 0; a < 4; ++a) {
                    int mt = a, pt = a;
                    assign[peel] = a;
                    double tmp = trait[a];
                    if (tmp == 0.0) continue;
                    for (int q = p->prev_off[k]; q < p->prev_off[k + 1]; ++q) {
                        int jj = p->prev[q];
                        tmp *= mat[jj][prev_index(p, jj, assign)];
                    }
                    double child_prob = 1.0;
                    for (int q = 0; q < c; ++q) {
                        int ch = cs[q];
                        if (!(p->mother[ch] == peel || p->father[ch] == peel)) continue;
                        int kt = assign[ch];
                        if (p->mother[ch] == peel) pt = assign[p->father[ch]];
                        else mt = assign[p->mother[ch]];
                        double ctmp = 0.0;
                        for (int i = 0; i < 2; ++i)
                            for (int j = 0; j < 2; ++j) {
                                if (phased_trait(mt, pt, i, j) != kt) continue;
                                ctmp += (t->dg == NULL) ? 0.25 : 0.25 * trait_rec(p, t, ch, i, j);
                            }
                        child_prob *= ctmp;
                    }
                    tmp *= child_prob;
                    total += tmp;
                }
            } else {
                for (int i = 0; i < 4; ++i) {
                    assign[peel] = i;
                    double tmp = trait[i];
                    if (tmp == 0.0) continue;
                    for (int q = p->prev_off[k]; q < p->prev_off[k + 1]; ++q) {
                        int jj = p->prev[q];
                        tmp *= mat[jj][prev_index(p, jj, assign)];
                    }
                    total += tmp;
                }
            }
            mat[k][cell] = total;
            if (total > vmax) vmax = total;
        }
        if (esum && vmax > 0.0) {
            int e;
            frexp(vmax, &e);
            for (int cell = 0; cell < ipow4(c); ++cell) mat[k][cell] = ldexp(mat[k][cell], -e);
            *esum += e;
        }
    }
    (void)N;
    return mat[p->K - 1][0];
}

static const double LOGZERO = -DBL_MAX;

static double log_sum(double a, double b) {  /* logarithms.cc:14-25 */
    if (a == LOGZERO) return b;
    if (b == LOGZERO) return a;
    return log(exp(b - a) + 1) + a;
}

int slo_lod(const slo_problem* p, const int32_t* dgs, int n_dgs, double* raw, uint32_t* count,
            double* trait_prob) {
    return slo_lod_ex(p, dgs, n_dgs, raw, count, trait_prob, 0);
}

/* zero_ok = 0: stop at a zero trait likelihood as Peeler::process does
 * (peeler.cc:89-92).  zero_ok = 1: count it as a zero term of the log-sum
 * (the value -DBL_MAX, which log_sum skips). */
int slo_lod_ex(const slo_problem* p, const int32_t* dgs, int n_dgs, double* raw, uint32_t* count,
               double* trait_prob, int zero_ok) {
    return slo_lod_range(p, dgs, n_dgs, 0, p->M - 1, 0, raw, count, trait_prob, zero_ok);
}

/* log of a peel's value: plain, or rescaled (log of the scaled value plus
   esum ln 2) */
static double peel_log(double r, const long* esum) {
    return esum ? log(r) + (double)*esum * 0.69314718055994530942 : log(r);
}

int slo_lod_range(const slo_problem* p, const int32_t* dgs, int n_dgs, int l0, int l1, int rescale, double* raw,
                  uint32_t* count, double* trait_prob, int zero_ok) {
    int K = p->K, M = p->M, n = p->n_lod, N = p->N;
    if (l0 < 0 || l1 > M - 1 || l0 > l1) return -2;
    double** mat = (double**)calloc(K, sizeof(double*));
    for (int k = 0; k < K; ++k) mat[k] = (double*)calloc(ipow4(cut_len(p, k)), sizeof(double));
    int* assign = (int*)malloc(sizeof(int) * N);
    long es = 0;
    long* esum = rescale ? &es : NULL;
    tctx t;
    memset(&t, 0, sizeof(t));
    t.dg = NULL;
    double tp = peel_log(trait_peel(p, &t, mat, assign, esum), esum);  /* peeler.cc:65-73 */
    int nscores = (l1 - l0) * n;
    unsigned char* init = (unsigned char*)calloc(nscores > 0 ? nscores : 1, 1);
    int nnf = N - p->F;
    double marker_trans = log(0.5) * (2 * nnf);  /* descent_graph.cc:22 */
    uint32_t cnt = 0;
    int rc = 0;
    size_t stride = (size_t)2 * N * M;
    for (int d = 0; d < n_dgs; ++d) {
        const int32_t* dg = dgs + d * stride;
        ++cnt;
        for (int l = l0; l < l1; ++l) {
            /* DescentGraph::get_recombination_prob (descent_graph.cc:212-242) */
            double lt = log(p->theta[l]), la = log(1.0 - p->theta[l]);
            double rec = 0.0;
            for (int i = p->F; i < N; ++i)
                for (int j = 0; j < 2; ++j)
                    rec += (dgget(p, dg, i, l, j) != dgget(p, dg, i, l + 1, j)) ? lt : la;
            for (int o = 0; o < n; ++o) {
                /* TraitRfunction::set_thetas (trait_rfunction.h:50-56) */
                t.dg = dg;
                t.locus = l;
                t.th = p->partial[l] * (o + 1);
                t.an = 1.0 - t.th;
                t.th2 = p->partial[l] * (n + 1 - (o + 1));
                t.an2 = 1.0 - t.th2;
                double r = trait_peel(p, &t, mat, assign, esum);
                if (r <= 0.0 && !zero_ok) { rc = -1; goto out; }
                double prob = r > 0.0 ? peel_log(r, esum) - rec - marker_trans : -DBL_MAX;
                int idx = (l - l0) * n + o;
                raw[idx] = init[idx] ? log_sum(prob, raw[idx]) : prob;
                init[idx] = 1;
            }
        }
    }
out:
    *count = cnt;
    *trait_prob = tp;
    for (int k = 0; k < K; ++k) free(mat[k]);
    free(mat);
    free(assign);
    free(init);
    return rc;
}

double slo_loglik(const slo_problem* p, const int32_t* dg) {
    int M = p->M, N = p->N;
    double marker_trans = log(0.5) * (2 * (N - p->F));
    /* DescentGraph::_recombination_prob (descent_graph.cc:200-210): a sum of the
       per-interval sums of get_recombination_prob (descent_graph.cc:212-242) */
    double rec = 0.0;
    for (int l = 0; l < M - 1; ++l) {
        double lt = log(p->theta[l]), la = log(1.0 - p->theta[l]);
        double r = 0.0;
        for (int i = p->F; i < N; ++i)
            for (int j = 0; j < 2; ++j)
                r += (dgget(p, dg, i, l, j) != dgget(p, dg, i, l + 1, j)) ? lt : la;
        rec += r;
    }
    fws f;
    fws_init(p, &f);
    double prior = 0.0;
    for (int l = 0; l < M; ++l) {
        fag_edges(p, dg, l, &f, -1, 0);
        double x = fag_like(p, l, &f);
        if (x == 0.0) { prior = LOGZERO; break; }
        prior += log(x);
    }
    fws_free(&f);
    if (prior == LOGZERO) return LOGZERO;
    return (marker_trans + rec) + prior;
}

/* ---------------------------------------------------------------------------
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11), the counter-based generator the device driver
 * uses; restated here so host replays can reproduce device draws.
 * ------------------------------------------------------------------------- */
double slo_philox_uniform(uint64_t key, uint64_t c_hi, uint64_t c_lo) {
    uint32_t c0 = (uint32_t)c_lo, c1 = (uint32_t)(c_lo >> 32);
    uint32_t c2 = (uint32_t)c_hi, c3 = (uint32_t)(c_hi >> 32);
    uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    uint64_t hi = c0 >> 5, lo = c1 >> 6;
    return (double)(hi * 67108864ull + lo) * (1.0 / 9007199254740992.0);
}


/* ---------------------------------------------------------------------------
 * Sequential imputation (LocusSampler::start_from, locus_sampler2.cc:214-241):
 * the starting locus with no neighbours, then leftwards using the right
 * neighbour only, then rightwards using the left neighbour only; the weight is
 * the sum of log(root) over the steps.  Draws are consumed in one sequence.
 * ------------------------------------------------------------------------- */
int slo_si(const slo_problem* p, int32_t* dg, int start, const double* u, int n_u, int* n_used, double* weight) {
    int used = 0, rc = 0, M = p->M;
    double wsum = 0.0;
    for (int v = 0; v < M; ++v) {
        int l = v == 0 ? start : (v <= start ? start - v : v);
        if (v == 0) { g_has_left = 0; g_has_right = 0; }
        else if (v <= start) { g_has_left = 0; g_has_right = l != M - 1; }
        else { g_has_left = l != 0; g_has_right = 0; }
        int n = 0;
        rc = slo_lstep(p, dg, l, u + used, n_u - used, &n);
        used += n;
        if (rc) break;
        wsum += log(g_last_root);
    }
    g_has_left = g_has_right = -1;
    *n_used = used;
    *weight = wsum;
    return rc;
}
