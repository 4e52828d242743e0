// TEST INFRASTRUCTURE ONLY (part of the oracle, never shipped or measured).
//
// C entry points over the reference's own CPU classes, compiled here from the
// reference sources (see oracle/Makefile) into oracle/_ref/libswiftref.so.
// Used only to pin the C restatement in oracle/sl_oracle.c and to write the
// golden fixtures under tests/golden/.  Descent graphs cross this boundary in
// the reference's internal layout: int32 [locus][person][2], offset
// 2N*locus + 2*person + parent (descent_graph.h:35-37).

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "descent_graph.h"
#include "disease_model.h"
#include "elimination.h"
#include "genetic_map.h"
#include "linkage_parser.h"
#include "locus_sampler2.h"
#include "lod_score.h"
#include "linkage_writer.h"
#include "map_parser.h"
#include "meiosis_sampler.h"
#include "pedigree.h"
#include "pedigree_parser.h"
#include "peel_sequence_generator.h"
#include "peeler.h"
#include "person.h"
#include "sequential_imputation.h"

using namespace std;

extern "C" void stub_seed(unsigned int seed);
extern "C" void stub_arm(const double* buf, int len);
extern "C" int stub_disarm();

struct RefState {
    GeneticMap map;
    DiseaseModel dm;
    vector<Pedigree> peds;
    Pedigree* ped;
    PeelSequenceGenerator* psg;
    LocusSampler* ls;
    MeiosisSampler* ms;
    GenotypeElimination* ge;
    bool sex_linked;
    RefState(int n_lod) : map(n_lod), dm(), peds(), ped(0), psg(0), ls(0), ms(0), ge(0), sex_linked(false) {}
};

extern "C" void* ref_load(const char* pedf, const char* mapf, const char* datf, int n_lod,
                          int peel_iters, unsigned seed) {
    RefState* s = new RefState(n_lod);
    stub_seed(seed);
    MapParser mp(mapf, s->map);
    if (!mp.parse()) return 0;
    LinkageParser lp(datf, s->map, s->dm);
    if (!lp.parse()) return 0;
    if (!s->map.sanity_check()) return 0;
    PedigreeParser pp(pedf, s->peds, s->dm, s->map);
    if (!pp.parse()) return 0;
    if (s->peds.size() != 1) return 0;
    s->ped = &s->peds[0];
    s->sex_linked = s->dm.is_sexlinked();
    s->psg = new PeelSequenceGenerator(s->ped, &s->map, s->sex_linked, false);
    s->psg->build_peel_sequence(peel_iters);
    s->ls = new LocusSampler(s->ped, &s->map, s->psg, 0, s->sex_linked);
    s->ms = new MeiosisSampler(s->ped, &s->map, s->sex_linked);
    s->ge = new GenotypeElimination(s->ped, s->sex_linked);
    s->ge->elimination();
    return s;
}

extern "C" void ref_free(void* h) {
    RefState* s = (RefState*)h;
    delete s->ls;
    delete s->ms;
    delete s->ge;
    delete s->psg;
    delete s;
}

extern "C" int ref_dims(void* h, int* N, int* F, int* M, int* K, int* n_lod, int* sex_linked) {
    RefState* s = (RefState*)h;
    *N = s->ped->num_members();
    *F = s->ped->num_founders();
    *M = s->map.num_markers();
    *K = s->psg->get_peel_order().size();
    *n_lod = s->map.get_lodscore_count();
    *sex_linked = s->sex_linked ? 1 : 0;
    return 0;
}

extern "C" int ref_pedigree(void* h, int* mother, int* father, int* sex, int* typed, int* affection,
                            unsigned char* genotypes, double* disease_prob, double* trait_prior,
                            int* n_children_out) {
    RefState* s = (RefState*)h;
    int N = s->ped->num_members();
    int M = s->map.num_markers();
    for (int i = 0; i < N; ++i) {
        Person* p = s->ped->get_by_index(i);
        mother[i] = p->isfounder() ? -1 : (int)p->get_maternalid();
        father[i] = p->isfounder() ? -1 : (int)p->get_paternalid();
        sex[i] = (int)p->get_sex();
        typed[i] = p->istyped() ? 1 : 0;
        affection[i] = (int)p->get_affection();
        n_children_out[i] = p->num_children();
        for (int v = 0; v < 4; ++v) disease_prob[i * 4 + v] = p->get_disease_prob((enum phased_trait)v);
        for (int l = 0; l < M; ++l) {
            genotypes[(size_t)l * N + i] = (unsigned char)p->get_marker(l);
            for (int v = 0; v < 4; ++v)
                trait_prior[((size_t)l * N + i) * 4 + v] = p->get_trait_probability(l, (enum phased_trait)v);
        }
    }
    return 0;
}

extern "C" int ref_map(void* h, double* theta, double* minor, double* partial, double* gpos) {
    RefState* s = (RefState*)h;
    int M = s->map.num_markers();
    for (int i = 0; i < M; ++i) {
        minor[i] = s->map.get_minor(i);
        gpos[i] = s->map.get_marker(i).get_g_distance();
        if (i < M - 1) {
            theta[i] = s->map.get_theta(i);
            partial[i] = s->map.get_theta_partial_raw(i);
        }
    }
    return 0;
}

extern "C" int ref_disease(void* h, double* freq, double* pen) {
    RefState* s = (RefState*)h;
    *freq = s->dm.get_freq();
    for (int i = 0; i < 3; ++i) pen[i] = s->dm.get_penetrance((enum unphased_trait)i);
    return 0;
}

// ops are written padded: cutset[K][maxc], prev[K][maxc], children[K][maxc]
extern "C" int ref_ops(void* h, int maxc, int* type, int* peelnode, int* cutset_len, int* cutset,
                       int* prev_len, int* prev, int* child_len, int* children, int* n_lod_cells) {
    RefState* s = (RefState*)h;
    vector<PeelOperation>& ops = s->psg->get_peel_order();
    for (size_t k = 0; k < ops.size(); ++k) {
        PeelOperation& op = ops[k];
        type[k] = (int)op.get_type();
        peelnode[k] = op.get_peelnode();
        vector<unsigned>& c = op.get_cutset();
        vector<unsigned>& p = op.get_prevfunctions();
        vector<unsigned>& ch = op.get_children();
        if ((int)c.size() > maxc || (int)p.size() > maxc || (int)ch.size() > maxc) return -1;
        cutset_len[k] = c.size();
        for (size_t i = 0; i < c.size(); ++i) cutset[k * maxc + i] = c[i];
        prev_len[k] = p.size();
        for (size_t i = 0; i < p.size(); ++i) prev[k * maxc + i] = p[i];
        child_len[k] = ch.size();
        for (size_t i = 0; i < ch.size(); ++i) children[k * maxc + i] = ch[i];
        n_lod_cells[k] = op.get_lod_indices()->size();
    }
    return 0;
}

extern "C" int ref_legal(void* h, unsigned char* legal) {
    RefState* s = (RefState*)h;
    int N = s->ped->num_members();
    int M = s->map.num_markers();
    for (int l = 0; l < M; ++l)
        for (int i = 0; i < N; ++i) {
            unsigned char m = 0;
            for (int v = 0; v < 4; ++v)
                if (s->ge->is_legal(i, l, v)) m |= (1u << v);
            legal[(size_t)l * N + i] = m;
        }
    return 0;
}

static void dg_in(RefState* s, DescentGraph& dg, const int* src) {
    memcpy(dg.get_internal_ptr(), src, dg.get_internal_size());
}

static void dg_out(RefState* s, DescentGraph& dg, int* dst) {
    memcpy(dst, dg.get_internal_ptr(), dg.get_internal_size());
}

extern "C" int ref_initial_dg(void* h, int si_iters, int* dg_out_buf, double* loglik) {
    RefState* s = (RefState*)h;
    DescentGraph dg(s->ped, &s->map, s->sex_linked);
    if (!dg.random_descentgraph()) return -1;
    SequentialImputation si(s->ped, &s->map, s->psg, s->sex_linked);
    si.parallel_run(dg, si_iters);
    *loglik = dg.get_likelihood();
    dg_out(s, dg, dg_out_buf);
    return 0;
}

extern "C" int ref_loglik(void* h, const int* dg_in_buf, double* loglik) {
    RefState* s = (RefState*)h;
    DescentGraph dg(s->ped, &s->map, s->sex_linked);
    dg_in(s, dg, dg_in_buf);
    *loglik = dg.get_likelihood();
    return 0;
}

// One sequential-imputation pass from `start` (LocusSampler::start_from,
// locus_sampler2.cc:214-241) with the injected draws; returns its weight.
extern "C" int ref_si(void* h, int* dg_io, int start, const double* u, int n_u, int* n_used, double* weight) {
    RefState* s = (RefState*)h;
    DescentGraph dg(s->ped, &s->map, s->sex_linked);
    dg_in(s, dg, dg_io);
    stub_arm(u, n_u);
    *weight = s->ls->start_from(dg, (unsigned)start);
    *n_used = stub_disarm();
    dg_out(s, dg, dg_io);
    return *n_used < 0 ? -1 : 0;
}

// Temper the map in place (GeneticMap::set_temperature, once per map) and
// rebuild the samplers on it, as a tempered MarkovChain holds them.
extern "C" int ref_set_temperature(void* h, double t) {
    RefState* s = (RefState*)h;
    s->map.set_temperature(t);
    delete s->ls;
    delete s->ms;
    s->ls = new LocusSampler(s->ped, &s->map, s->psg, 0, s->sex_linked);
    s->ms = new MeiosisSampler(s->ped, &s->map, s->sex_linked);
    return 0;
}

// get_likelihood2 under a copy of the map at MC3 temperature t, as
// MarkovChain::get_likelihood does for a tempered chain (markov_chain.h:122-124).
extern "C" int ref_loglik_tempered(void* h, const int* dg_in_buf, double t, double* loglik) {
    RefState* s = (RefState*)h;
    GeneticMap m(s->map);
    if (t != 1.0) m.set_temperature(t);
    DescentGraph dg(s->ped, &s->map, s->sex_linked);
    dg_in(s, dg, dg_in_buf);
    *loglik = dg.get_likelihood2(&m);
    return 0;
}

// One L-sampler step at `locus` (locus_sampler2.cc:128-159 after set_locus_minimal).
extern "C" int ref_lstep(void* h, int* dg_io, int locus, const double* u, int n_u, int* n_used) {
    RefState* s = (RefState*)h;
    DescentGraph dg(s->ped, &s->map, s->sex_linked);
    dg_in(s, dg, dg_io);
    s->ls->set_locus_minimal(locus);
    stub_arm(u, n_u);
    s->ls->step(dg, locus);
    *n_used = stub_disarm();
    dg_out(s, dg, dg_io);
    return *n_used < 0 ? -1 : 0;
}

// One M-sweep: reset at meioses[0], then a step per meiosis in order
// (markov_chain.cc:345-351).  Each step draws from its own slice of M values.
extern "C" int ref_msweep(void* h, int* dg_io, const int* meioses, int n, const double* u,
                          int* n_used) {
    RefState* s = (RefState*)h;
    int M = s->map.num_markers();
    DescentGraph dg(s->ped, &s->map, s->sex_linked);
    dg_in(s, dg, dg_io);
    s->ms->reset(dg, meioses[0]);
    for (int j = 0; j < n; ++j) {
        stub_arm(u + (size_t)j * M, M);
        s->ms->step(dg, meioses[j]);
        n_used[j] = stub_disarm();
        if (n_used[j] < 0) return -1;
    }
    dg_out(s, dg, dg_io);
    return 0;
}

// LOD scoring of a set of descent graphs (peeler.cc:65-103, lod_score.h:74-105).
extern "C" int ref_lod(void* h, const int* dgs, int n_dgs, double* raw, unsigned* count,
                       double* trait_prob) {
    RefState* s = (RefState*)h;
    int M = s->map.num_markers();
    LODscores lod(&s->map);
    Peeler peeler(s->ped, &s->map, s->psg, &lod, s->sex_linked);
    double tp = peeler.calc_trait_prob();
    lod.set_trait_prob(tp);
    DescentGraph dg(s->ped, &s->map, s->sex_linked);
    size_t stride = dg.get_internal_size() / sizeof(int);
    for (int d = 0; d < n_dgs; ++d) {
        dg_in(s, dg, dgs + d * stride);
        for (int l = 0; l < M - 1; ++l) {
            peeler.set_locus(l);
            peeler.process(&dg);
        }
    }
    for (unsigned i = 0; i < lod.num_lodscores(); ++i) raw[i] = lod.get_raw(i);
    *count = lod.get_count();
    *trait_prob = tp;
    return 0;
}

// The reference's LOD table writer (LinkageWriter::write, linkage_writer.cc:
// 14-89) on given log-sums, count and log P(T) of the loaded family.
extern "C" int ref_write_table(void* h, const double* raw, unsigned count, double trait_prob, const char* path) {
    RefState* s = (RefState*)h;
    LODscores lod(&s->map);
    for (unsigned i = 0; i < lod.num_lodscores(); ++i) lod.set(i, raw[i]);
    lod.set_count(count);
    lod.set_trait_prob(trait_prob);
    vector<LODscores*> all(1, &lod);
    LinkageWriter w(&s->map, path, false);
    return w.write(all) ? 0 : -1;
}

extern "C" int ref_meiosis_order(void* h, int* out, int* n_out) {
    // non-ignorable meioses, in index order (markov_chain.cc:70-80)
    RefState* s = (RefState*)h;
    int F = s->ped->num_founders();
    int N = s->ped->num_members();
    int n = 0;
    for (int i = 0; i < 2 * (N - F); ++i) {
        Person* p = s->ped->get_by_index(F + i / 2);
        if (!p->safe_to_ignore_meiosis((enum parentage)(i % 2))) out[n++] = i;
    }
    *n_out = n;
    return 0;
}
