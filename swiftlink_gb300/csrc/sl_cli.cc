// swift_gb300: the `swift` program surface (main.cc, linkage_program.cc) over
// the library's C ABI.  LINKAGE ped/map/dat in, the per-position LOD table out
// (the format of LinkageWriter::write, linkage_writer.cc:14-89), the same
// options; every pedigree runs on the GPU, all pedigrees in one batch.
//
// Reading the inputs restates the reference's parsers: PedigreeParser
// (pedigree_parser.cc: famid id father mother sex affection, then allele pairs
// "0 0" missing, "1" = A major, "2" = B minor), MapParser (map_parser.cc:
// chromosome, genetic position in cM, name), LinkageParser (linkage_parser.cc:
// the header lines, the affection-status trait locus with its frequencies,
// one liability class of three penetrances, then the numbered-allele markers
// with two frequencies each, the recombination lines ignored because theta is
// recomputed from the map, genetic_map.cc:14-64).  Members are put founders
// first by std::sort with the reference's comparator (Pedigree::
// _reorder_family, pedigree.cc:154-161), so the internal order is the same.
#include <getopt.h>

#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/swiftlink_gb300.h"

namespace {

struct Options {
    std::string ped, map, dat, out = "swiftlink.out", trace_prefix = "trace", seeds, dump, write_from;
    int iterations = 50000, burnin = 50000, si = 1000, period = 10, lods = 5, runs = 1;
    int chains = 1, exchange = 10;   // MC3 (defaults.h:9, 12)
    double lprob = 0.5;
    std::vector<double> temps;
    bool trace = false, affected_only = false, verbose = false, exact = false, mc3 = false, generic_ls = false,
         compiled_ls = false;
};

std::vector<std::string> tokens(const std::string& line) {
    std::vector<std::string> t;
    std::istringstream ss(line);
    std::string w;
    while (ss >> w) {
        if (w[0] == '#') break;
        t.push_back(w);
    }
    return t;
}

bool read_lines(const std::string& path, std::vector<std::string>& lines) {
    std::ifstream f(path);
    if (!f) {
        fprintf(stderr, "error: could not open '%s'\n", path.c_str());
        return false;
    }
    std::string l;
    while (std::getline(f, l)) lines.push_back(l);
    return true;
}

struct Member {
    std::string id, father, mother;
    int sex = 0, affection = 0;
    std::vector<int> geno;   // UNTYPED 0, HETERO 1, HOMOZ_A 2, HOMOZ_B 3
    bool founder_str() const { return father == "0" && mother == "0"; }
    bool operator<(const Member& p) const { return founder_str() && !p.founder_str(); }
};

struct Family {
    std::string id;
    std::vector<Member> members;
};

struct Model {
    int n_loci = 0;
    double freq = 0.0;
    double pen[3] = {0, 0, 1};
    std::vector<double> minor;
};

struct Marker {
    std::string name;
    double g;   // Morgans
};

// PedigreeParser::_parse_genotype (pedigree_parser.cc)
bool parse_genotype(const std::string& a, const std::string& b, int& g) {
    if (a == "0" || b == "0") { g = 0; return true; }
    if (a == b) {
        if (a == "1") { g = 2; return true; }
        if (a == "2") { g = 3; return true; }
        return false;
    }
    if ((a == "1" && b == "2") || (a == "2" && b == "1")) { g = 1; return true; }
    return false;
}

bool parse_ped(const std::string& path, std::vector<Family>& fams) {
    std::vector<std::string> lines;
    if (!read_lines(path, lines)) return false;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        const auto t = tokens(lines[ln]);
        if (t.empty()) continue;
        if (t.size() < 6 || t.size() % 2) {
            fprintf(stderr, "error: %s, line %d: expected 6 fields and allele pairs\n", path.c_str(), (int)ln + 1);
            return false;
        }
        Member m;
        m.id = t[1];
        m.father = t[2];
        m.mother = t[3];
        if (t[4] != "0" && t[4] != "1" && t[4] != "2") {
            fprintf(stderr, "error: %s, line %d: bad sex \"%s\" (column 5)\n", path.c_str(), (int)ln + 1, t[4].c_str());
            return false;
        }
        if (t[5] != "0" && t[5] != "1" && t[5] != "2") {
            fprintf(stderr, "error: %s, line %d: bad affection status \"%s\" (column 6)\n", path.c_str(), (int)ln + 1,
                    t[5].c_str());
            return false;
        }
        m.sex = t[4][0] - '0';
        m.affection = t[5][0] - '0';
        for (size_t k = 6; k < t.size(); k += 2) {
            int g;
            if (!parse_genotype(t[k], t[k + 1], g)) {
                fprintf(stderr, "error: %s, line %d: error parsing genotype %d\n", path.c_str(), (int)ln + 1,
                        (int)(k - 6) / 2 + 1);
                return false;
            }
            m.geno.push_back(g);
        }
        Family* f = nullptr;
        for (auto& x : fams)
            if (x.id == t[0]) f = &x;
        if (!f) {
            fams.push_back(Family{t[0], {}});
            f = &fams.back();
        }
        for (auto& x : f->members)
            if (x.id == m.id) {
                fprintf(stderr, "error: %s, line %d: person %s appears twice\n", path.c_str(), (int)ln + 1, m.id.c_str());
                return false;
            }
        f->members.push_back(m);
    }
    if (fams.empty()) {
        fprintf(stderr, "error: %s contains no families\n", path.c_str());
        return false;
    }
    return true;
}

bool parse_map(const std::string& path, std::vector<Marker>& map) {
    std::vector<std::string> lines;
    if (!read_lines(path, lines)) return false;
    for (size_t ln = 0; ln < lines.size(); ++ln) {
        const auto t = tokens(lines[ln]);
        if (t.empty()) continue;
        if (t.size() < 3) {
            fprintf(stderr, "error: %s, line %d: expected chromosome, genetic position, marker name\n", path.c_str(),
                    (int)ln + 1);
            return false;
        }
        std::istringstream ss(t[1]);
        double g;
        if ((ss >> g).fail() || g < 0.0) {
            fprintf(stderr, "error: %s, line %d: bad genetic position '%s'\n", path.c_str(), (int)ln + 1, t[1].c_str());
            return false;
        }
        map.push_back({t[2], g / 100.0});   // MapParser: cM to Morgans
    }
    return map.size() > 1;
}

std::vector<double> doubles(const std::vector<std::string>& t) {
    std::vector<double> v;
    for (const auto& w : t) {
        std::istringstream ss(w);
        double d;
        if (!(ss >> d).fail()) v.push_back(d);
    }
    return v;
}

bool parse_dat(const std::string& path, Model& m, bool& sexlinked) {
    std::vector<std::string> raw, lines;
    if (!read_lines(path, raw)) return false;
    for (auto& l : raw)
        if (!tokens(l).empty()) lines.push_back(l);
    if (lines.size() < 3) return false;
    auto h = tokens(lines[0]);
    if (h.size() != 4) {
        fprintf(stderr, "error: expected 4 fields on line 1 of LINKAGE dat file (read %d)\n", (int)h.size());
        return false;
    }
    m.n_loci = atoi(h[0].c_str());
    sexlinked = h[2] == "1";
    size_t ln = 3;
    bool trait = false;
    for (int locus = 0; locus < m.n_loci; ++locus) {
        if (ln >= lines.size()) return false;
        auto t = tokens(lines[ln++]);
        const int code = atoi(t[0].c_str());
        if (ln >= lines.size()) return false;
        const auto af = doubles(tokens(lines[ln++]));
        if (af.size() != 2) {
            fprintf(stderr, "error: %s: only loci with 2 alleles are handled\n", path.c_str());
            return false;
        }
        if (af[0] + af[1] < 0.99) {
            fprintf(stderr, "error: %s: allele frequencies do not sum to 1.0\n", path.c_str());
            return false;
        }
        if (code == 1) {   // affection status: liability classes, then one line of penetrances
            if (locus != 0) {
                fprintf(stderr, "error: %s: trait marker must be the first marker in linkage file\n", path.c_str());
                return false;
            }
            if (ln >= lines.size()) return false;
            const int classes = atoi(tokens(lines[ln++])[0].c_str());
            if (classes != 1) fprintf(stderr, "Apologises: \"more than one liability class\" not supported\n");
            if (ln >= lines.size()) return false;
            const auto pen = doubles(tokens(lines[ln++]));
            if (pen.size() != 3) {
                fprintf(stderr, "error: %s: liability classes should contain three numbers\n", path.c_str());
                return false;
            }
            for (int k = 0; k < 3; ++k) m.pen[k] = pen[k];
            m.freq = af[1];
            trait = true;
        } else if (code == 3) {
            m.minor.push_back(af[1]);
        } else {
            fprintf(stderr, "Apologises: marker code %d not supported\n", code);
            return false;
        }
    }
    if (!trait) {
        fprintf(stderr, "error: %s: did not read trait marker\n", path.c_str());
        return false;
    }
    return true;
}

// log_sum (logarithms.cc:14-25), LOG_ZERO = -DBL_MAX
double log_sum(double a, double b) {
    if (a == -DBL_MAX) return b;
    if (b == -DBL_MAX) return a;
    return std::log(std::exp(b - a) + 1) + a;
}

bool csv_doubles(const char* s, std::vector<double>& v) {
    std::stringstream ss(s);
    std::string w;
    v.clear();
    while (std::getline(ss, w, ',')) {
        char* end;
        const double x = strtod(w.c_str(), &end);
        if (w.empty() || *end != '\0' || !(x >= 0.0 && x <= 1.0)) return false;
        v.push_back(x);
    }
    return !v.empty();
}

double haldane(double m) { return 0.5 * (1.0 - std::exp(-2.0 * m)); }
double inverse_haldane(double r) { return -0.5 * std::log(1 - (2 * r)); }

// DiseaseModel::get_apriori_prob2 / get_penetrance_prob2 (disease_model.cc:
// 139-187) through Person::_init_probs (person.cc:85-119), autosomal; phased
// order UU, AA, AU, UA.
void disease_prob(const Model& m, bool founder, int affection, double* out) {
    const double q = m.freq;
    const double prior[3] = {(1.0 - q) * (1.0 - q), q * (1.0 - q), q * q};
    const int unph[4] = {0, 2, 1, 1};
    for (int v = 0; v < 4; ++v) {
        const int t = unph[v];
        const double pen = m.pen[t];
        if (founder) {
            if (affection == 2) out[v] = prior[t] * pen;
            else if (affection == 1) out[v] = prior[t] * (1.0 - pen);
            else out[v] = (prior[t] * pen) + (prior[t] * (1.0 - pen));
        } else {
            out[v] = affection == 2 ? pen : (affection == 1 ? 1.0 - pen : 0.25);
        }
    }
}

// One family as the library's problem.
struct Problem {
    int N = 0, F = 0;
    std::vector<int32_t> mother, father, sex, affection, op_type, op_peel, cut_off, cut, prev_off, prev, ch_off, ch;
    std::vector<uint8_t> typed, geno;
    std::vector<double> dprob;
};

bool build_family(const Family& fam, const Model& model, const std::vector<Marker>& map, bool affected_only,
                  Problem& p) {
    std::vector<Member> mem = fam.members;
    std::sort(mem.begin(), mem.end());   // founders first, as the reference's std::sort leaves them
    const int N = (int)mem.size(), M = (int)map.size();
    std::map<std::string, int> idx;
    for (int i = 0; i < N; ++i) idx[mem[i].id] = i;
    p.N = N;
    p.mother.assign(N, -1);
    p.father.assign(N, -1);
    p.sex.assign(N, 0);
    p.affection.assign(N, 0);
    p.typed.assign(N, 0);
    p.geno.assign((size_t)M * N, 0);
    p.dprob.assign((size_t)4 * N, 0.0);
    for (int i = 0; i < N; ++i) {
        const Member& m = mem[i];
        if ((int)m.geno.size() != M) {
            fprintf(stderr, "error: family %s, person %s has %d genotypes, the map %d markers\n", fam.id.c_str(),
                    m.id.c_str(), (int)m.geno.size(), M);
            return false;
        }
        if (!m.founder_str()) {
            if (!idx.count(m.mother) || !idx.count(m.father)) {
                fprintf(stderr, "error: family %s, person %s: a parent is missing\n", fam.id.c_str(), m.id.c_str());
                return false;
            }
            p.mother[i] = idx[m.mother];
            p.father[i] = idx[m.father];
        } else {
            p.F++;
        }
        p.sex[i] = m.sex;
        p.affection[i] = (affected_only && m.affection != 2) ? 0 : m.affection;
        for (int l = 0; l < M; ++l) {
            p.geno[(size_t)l * N + i] = (uint8_t)m.geno[l];
            if (m.geno[l]) p.typed[i] = 1;
        }
        disease_prob(model, m.founder_str(), p.affection[i], &p.dprob[(size_t)4 * i]);
    }
    for (int i = 0; i < p.F; ++i)
        if (!mem[i].founder_str()) return false;
    const int cap = N * N + 16;
    p.op_type.assign(N, 0);
    p.op_peel.assign(N, 0);
    p.cut_off.assign(N + 1, 0);
    p.prev_off.assign(N + 1, 0);
    p.ch_off.assign(N + 1, 0);
    p.cut.assign(cap, 0);
    p.prev.assign(cap, 0);
    p.ch.assign(cap, 0);
    if (sl_peel_sequence(N, p.mother.data(), p.father.data(), cap, p.op_type.data(), p.op_peel.data(),
                         p.cut_off.data(), p.cut.data(), p.prev_off.data(), p.prev.data(), p.ch_off.data(),
                         p.ch.data()) != SL_OK) {
        fprintf(stderr, "error: family %s: no peel sequence\n", fam.id.c_str());
        return false;
    }
    return true;
}

// The problem tables as text, one block per family (no device needed):
// "family ID N F M", then one named line per table, values in internal order.
bool dump_problems(const std::string& path, const std::vector<Family>& fams, const std::vector<Problem>& probs,
                   const std::vector<Marker>& map, const Model& model, const std::vector<double>& theta,
                   const std::vector<double>& partial) {
    FILE* f = fopen(path.c_str(), "w");
    if (!f) {
        fprintf(stderr, "error: could not open '%s'\n", path.c_str());
        return false;
    }
    auto ints = [&](const char* name, const std::vector<int32_t>& v) {
        fprintf(f, "%s", name);
        for (int32_t x : v) fprintf(f, " %d", x);
        fprintf(f, "\n");
    };
    auto reals = [&](const char* name, const std::vector<double>& v) {
        fprintf(f, "%s", name);
        for (double x : v) fprintf(f, " %.17g", x);
        fprintf(f, "\n");
    };
    const int M = (int)map.size();
    std::vector<double> gpos(M);
    for (int i = 0; i < M; ++i) gpos[i] = map[i].g;
    for (size_t k = 0; k < fams.size(); ++k) {
        const Problem& p = probs[k];
        std::vector<Member> mem = fams[k].members;
        std::sort(mem.begin(), mem.end());
        fprintf(f, "family %s %d %d %d\nids", fams[k].id.c_str(), p.N, p.F, M);
        for (const Member& m : mem) fprintf(f, " %s", m.id.c_str());
        fprintf(f, "\n");
        ints("mother", p.mother);
        ints("father", p.father);
        ints("sex", p.sex);
        ints("affection", p.affection);
        ints("typed", std::vector<int32_t>(p.typed.begin(), p.typed.end()));
        ints("genotypes", std::vector<int32_t>(p.geno.begin(), p.geno.end()));
        reals("disease_prob", p.dprob);
        reals("theta", theta);
        reals("partial", partial);
        reals("minor", model.minor);
        reals("gpos", gpos);
        reals("model", {model.freq, model.pen[0], model.pen[1], model.pen[2]});
        ints("op_type", p.op_type);
        ints("op_peel", p.op_peel);
    }
    fclose(f);
    return true;
}

// The LOD table in LinkageWriter::write's format (linkage_writer.cc:14-89):
// a header, then per marker interval the marker's name and position (cM) and
// one line per LOD position with its position, the LOD summed over families
// and, with more than one family, each family's LOD; the last marker closes.
// lod[f][(M-1) n] are the families' LODs, (raw - log count - P(T)) / log 10.
bool write_table(const Options& o, const std::vector<Marker>& map, const std::vector<double>& partial,
                 const std::vector<std::vector<double>>& lod) {
    const int M = (int)map.size(), n = o.lods;
    std::ofstream out(o.out, std::ios::out | std::ios::trunc);
    if (!out) {
        fprintf(stderr, "error: could not open linkage output file \"%s\"\n", o.out.c_str());
        return false;
    }
    auto gpos = [&](int i, int off) { return map[i].g + (off ? inverse_haldane(partial[i] * off) : 0.0); };
    out << "marker\tposition\tlod\n";
    for (int i = 0; i + 1 < M; ++i) {
        out << map[i].name << "\t" << 100.0 * gpos(i, 0) << "\n";
        for (int j = 0; j < n; ++j) {
            double t = lod[0][(size_t)i * n + j];
            for (size_t k = 1; k < lod.size(); ++k) t += lod[k][(size_t)i * n + j];
            std::stringstream ss;
            ss << "-\t" << 100 * gpos(i, j + 1) << "\t" << t;
            if (lod.size() > 1)
                for (size_t k = 0; k < lod.size(); ++k) ss << "\t" << lod[k][(size_t)i * n + j];
            ss << "\n";
            out << ss.str();
            if (o.verbose) fprintf(stderr, "%s", ss.str().c_str());
        }
    }
    out << map[M - 1].name << "\t" << 100.0 * gpos(M - 1, 0) << "\n";
    return true;
}

// -W: the families' log-sums, counts and log P(T) from a file, as LODs.
bool read_logsums(const std::string& path, size_t nfam, size_t npos, std::vector<std::vector<double>>& lod) {
    std::ifstream f(path);
    if (!f) {
        fprintf(stderr, "error: could not open '%s'\n", path.c_str());
        return false;
    }
    lod.assign(nfam, std::vector<double>(npos));
    for (size_t k = 0; k < nfam; ++k) {
        double count = 0, tp = 0;
        if (!(f >> count >> tp) || count < 1) {
            fprintf(stderr, "error: '%s': family %zu: bad count or P(T)\n", path.c_str(), k + 1);
            return false;
        }
        for (size_t i = 0; i < npos; ++i) {
            double raw;
            if (!(f >> raw)) {
                fprintf(stderr, "error: '%s': family %zu: %zu of %zu log-sums\n", path.c_str(), k + 1, i, npos);
                return false;
            }
            lod[k][i] = (raw - std::log(count) - tp) / std::log(10.0);
        }
    }
    return true;
}

void usage(const char* prog) {
    fprintf(stderr,
            "Usage: %s -p pedfile -m mapfile -d datfile [options]\n"
            "  -o FILE   --output=FILE             (default = swiftlink.out)\n"
            "  -i NUM    --iterations=NUM          (default = 50000)\n"
            "  -b NUM    --burnin=NUM              (default = 50000)\n"
            "  -s NUM    --sequentialimputation=NUM (default = 1000)\n"
            "  -x NUM    --scoringperiod=NUM       (default = 10)\n"
            "  -l FLOAT  --lsamplerprobability=FLOAT (default = 0.5)\n"
            "  -n NUM    --lodscores=NUM           (default = 5)\n"
            "  -R NUM    --runs=NUM                (default = 1; run as replicate chains on the device)\n"
            "  -T        --trace, -P PREFIX --traceprefix=PREFIX (default = trace)\n"
            "  -c NUM    --cores=NUM               (accepted; the work runs on the GPU)\n"
            "  -g        --gpu                     (accepted; always on)\n"
            "  -q NUM    --peelseqiter=NUM         (accepted; the peel sequence search is the library's)\n"
            "  -r FILE   --randomseeds=FILE        (the first integer seeds the device streams)\n"
            "  -a        --affectedonly, -v --verbose, -h --help\n"
            "  -M        --mcmcmc                  (MC3: -z tempered chains per run, exchanges every -y iterations)\n"
            "  -z NUM    --chains=NUM              (default = 1)\n"
            "  -y NUM    --exchangeperiod=NUM      (default = 10)\n"
            "  -t LIST   --temperatures=LIST       (comma separated, the first 1.0; default 1 / (1 + 0.001 2^i))\n"
            "  -E        --exact                   (FP64 samplers and LOD, the reference's arithmetic)\n"
            "  -G        --genericls               (the generic L-sampler, lanes per task by timing: the default)\n"
            "  -J        --compiledls              (long runs: also compile the L-sampler for each pedigree)\n"
            "  -D FILE   --dumpproblem=FILE        (write the problem tables of every family and stop)\n"
            "  -W FILE   --writetable=FILE         (write the LOD table from FILE's per-family log-sums and stop:\n"
            "                                       per family a line \"count log_P(T)\", then (M-1)*n raw values)\n",
            prog);
}

bool to_int(const char* s, int& v) {
    char* end;
    errno = 0;
    const long x = strtol(s, &end, 10);
    if (errno || *s == '\0' || *end != '\0' || x < INT32_MIN || x > INT32_MAX) return false;
    v = (int)x;
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    static struct option longopts[] = {
        {"pedigree", required_argument, 0, 'p'},  {"map", required_argument, 0, 'm'},
        {"dat", required_argument, 0, 'd'},       {"output", required_argument, 0, 'o'},
        {"iterations", required_argument, 0, 'i'}, {"burnin", required_argument, 0, 'b'},
        {"sequentialimputation", required_argument, 0, 's'}, {"scoringperiod", required_argument, 0, 'x'},
        {"lsamplerprobability", required_argument, 0, 'l'}, {"lodscores", required_argument, 0, 'n'},
        {"runs", required_argument, 0, 'R'},      {"trace", no_argument, 0, 'T'},
        {"traceprefix", required_argument, 0, 'P'}, {"cores", required_argument, 0, 'c'},
        {"gpu", no_argument, 0, 'g'},             {"peelseqiter", required_argument, 0, 'q'},
        {"randomseeds", required_argument, 0, 'r'}, {"affectedonly", no_argument, 0, 'a'},
        {"sexlinked", no_argument, 0, 'X'},       {"elod", no_argument, 0, 'e'},
        {"verbose", no_argument, 0, 'v'},         {"help", no_argument, 0, 'h'},
        {"exact", no_argument, 0, 'E'},           {"dumpproblem", required_argument, 0, 'D'},
        {"genericls", no_argument, 0, 'G'},     {"compiledls", no_argument, 0, 'J'},     {"writetable", required_argument, 0, 'W'},
        {"mcmcmc", no_argument, 0, 'M'},          {"chains", required_argument, 0, 'z'},
        {"exchangeperiod", required_argument, 0, 'y'}, {"temperatures", required_argument, 0, 't'},
        {"frequency", required_argument, 0, 'f'}, {"penetrance", required_argument, 0, 'k'},
        {"replicates", required_argument, 0, 'u'}, {"separation", required_argument, 0, 'w'},
        {0, 0, 0, 0}};
    int ch, ignored;
    while ((ch = getopt_long(argc, argv, "p:m:d:o:i:b:s:x:l:n:R:TP:c:gq:r:aXevhED:Mz:y:t:f:k:u:w:GJW:", longopts, nullptr)) != -1) {
        switch (ch) {
            case 'p': o.ped = optarg; break;
            case 'm': o.map = optarg; break;
            case 'd': o.dat = optarg; break;
            case 'o': o.out = optarg; break;
            case 'i': if (!to_int(optarg, o.iterations)) { fprintf(stderr, "option '-i' requires an int\n"); return 1; } break;
            case 'b': if (!to_int(optarg, o.burnin)) { fprintf(stderr, "option '-b' requires an int\n"); return 1; } break;
            case 's': if (!to_int(optarg, o.si)) { fprintf(stderr, "option '-s' requires an int\n"); return 1; } break;
            case 'x': if (!to_int(optarg, o.period)) { fprintf(stderr, "option '-x' requires an int\n"); return 1; } break;
            case 'n': if (!to_int(optarg, o.lods)) { fprintf(stderr, "option '-n' requires an int\n"); return 1; } break;
            case 'R': if (!to_int(optarg, o.runs)) { fprintf(stderr, "option '-R' requires an int\n"); return 1; } break;
            case 'l': o.lprob = atof(optarg); break;
            case 'T': o.trace = true; break;
            case 'P': o.trace_prefix = optarg; break;
            case 'c': case 'q': if (!to_int(optarg, ignored)) { fprintf(stderr, "option requires an int\n"); return 1; } break;
            case 'g': break;
            case 'r': o.seeds = optarg; break;
            case 'a': o.affected_only = true; break;
            case 'X': fprintf(stderr, "error: sex-linked analysis is not supported on the GPU\n"); return 1;
            case 'e': fprintf(stderr, "error: ELOD is not part of this program\n"); return 1;
            case 'v': o.verbose = true; break;
            case 'E': o.exact = true; break;
            case 'D': o.dump = optarg; break;
            case 'M': o.mc3 = true; break;
            case 'G': o.generic_ls = true; break;
            case 'J': o.compiled_ls = true; break;
            case 'W': o.write_from = optarg; break;
            case 'z': if (!to_int(optarg, o.chains) || o.chains < 1) { fprintf(stderr, "option '-z' requires an int > 0\n"); return 1; } break;
            case 'y': if (!to_int(optarg, o.exchange) || o.exchange < 1) { fprintf(stderr, "option '-y' requires an int > 0\n"); return 1; } break;
            case 't':
                if (!csv_doubles(optarg, o.temps)) {
                    fprintf(stderr, "temperatures must be comma delimited floats from 0.0 - 1.0 inclusive, e.g.: 1.0,0.9,0.8,0.7\n");
                    return 1;
                }
                break;
            case 'f': case 'k': case 'u': case 'w':
                fprintf(stderr, "error: ELOD is not part of this program\n");
                return 1;
            case 'h': usage(argv[0]); return 0;
            default: usage(argv[0]); return 1;
        }
    }
    if (o.ped.empty() || o.map.empty() || o.dat.empty()) {
        usage(argv[0]);
        return 1;
    }
    if (o.mc3 && !o.temps.empty() && ((int)o.temps.size() != o.chains || o.temps[0] != 1.0)) {
        fprintf(stderr, "error: -t needs one temperature per chain (-z), the first 1.0\n");
        return 1;
    }
    if (o.iterations < 1 || o.burnin < 0 || o.period < 1 || o.lods < 1 || o.runs < 1 || o.si < 0 ||
        !(o.lprob >= 0.0 && o.lprob <= 1.0)) {
        fprintf(stderr, "error: bad option values\n");
        return 1;
    }
    uint64_t seed = 20261205;
    if (!o.seeds.empty()) {
        std::ifstream f(o.seeds);
        unsigned long long s;
        if (!(f >> s)) { fprintf(stderr, "error: could not read a seed from '%s'\n", o.seeds.c_str()); return 1; }
        seed = s;
    }
    std::vector<Family> fams;
    std::vector<Marker> map;
    Model model;
    bool sexlinked = false;
    if (!parse_map(o.map, map) || !parse_dat(o.dat, model, sexlinked) || !parse_ped(o.ped, fams)) return 1;
    if (sexlinked) {
        fprintf(stderr, "error: sex-linked analysis is not supported on the GPU\n");
        return 1;
    }
    if (model.minor.size() != map.size()) {
        fprintf(stderr, "error: %d markers in the DAT file, %d in the MAP file\n", (int)model.minor.size(),
                (int)map.size());
        return 1;
    }
    const int M = (int)map.size(), n = o.lods;
    // GeneticMap::sanity_check: theta from the Haldane map, partial theta per position
    std::vector<double> theta(M - 1), partial(M - 1);
    for (int i = 0; i + 1 < M; ++i) {
        theta[i] = haldane(map[i + 1].g - map[i].g);
        if (theta[i] == 0.0) {
            fprintf(stderr, "error: recombination fraction between %s and %s is zero\n", map[i].name.c_str(),
                    map[i + 1].name.c_str());
            return 1;
        }
        partial[i] = haldane(inverse_haldane(theta[i]) / double(n + 1));
    }
    fprintf(stderr, "\nLinkage parameters:\n\tpenetrance = %.2f:%.2f:%.2f\n\ttrait freq = %.2e\n"
                    "\tburnin iterations = %d\n\tsampling iterations = %d\n\tsampling period = %d\n"
                    "\tlocus sampler prob = %.3f\n\tnumber of runs = %d\n\n",
            model.pen[0], model.pen[1], model.pen[2], model.freq, o.burnin, o.iterations, o.period, o.lprob, o.runs);
    std::vector<Problem> probs(fams.size());
    for (size_t f = 0; f < fams.size(); ++f)
        if (!build_family(fams[f], model, map, o.affected_only, probs[f])) return 1;
    if (!o.dump.empty()) return dump_problems(o.dump, fams, probs, map, model, theta, partial) ? 0 : 1;
    if (!o.write_from.empty()) {
        std::vector<std::vector<double>> lod;
        return read_logsums(o.write_from, fams.size(), (size_t)(M - 1) * n, lod) && write_table(o, map, partial, lod)
                   ? 0 : 1;
    }
    // Contexts: without MC3 one per family holding its -R runs as chains; with MC3
    // one per (family, run) holding the -z tempered chains, chain 0 at t = 1.
    struct Unit {
        size_t fam;
        int run;
        sl_ctx* ctx;
    };
    std::vector<Unit> units;
    std::vector<sl_ctx*> ctxs;
    const int per_ctx = o.mc3 ? o.chains : o.runs;
    std::vector<double> temps(per_ctx, 1.0);
    if (o.mc3)
        for (int i = 0; i < o.chains; ++i)   // Mc3::_init (mc3.cc:30-44)
            temps[i] = !o.temps.empty() ? o.temps[i] : (i == 0 ? 1.0 : 1.0 / (1.0 + (0.001 * std::pow(2.0, i))));
    int rc = 0;
    for (size_t f = 0; f < fams.size() && !rc; ++f) {
        Problem& p = probs[f];
        sl_problem_desc d{};
        d.n_members = p.N;
        d.n_founders = p.F;
        d.n_markers = M;
        d.lod_per_interval = n;
        d.mother = p.mother.data();
        d.father = p.father.data();
        d.sex = p.sex.data();
        d.typed = p.typed.data();
        d.genotypes = p.geno.data();
        d.disease_prob = p.dprob.data();
        d.theta = theta.data();
        d.partial_theta = partial.data();
        d.minor_freq = model.minor.data();
        d.n_ops = p.N;
        d.op_type = p.op_type.data();
        d.op_peelnode = p.op_peel.data();
        d.cutset_off = p.cut_off.data();
        d.cutset = p.cut.data();
        d.prev_off = p.prev_off.data();
        d.prev = p.prev.data();
        d.children_off = p.ch_off.data();
        d.children = p.ch.data();
        sl_options so{};
        so.n_chains = per_ctx;
        so.lod_precision = o.exact ? SL_LOD_FP64 : SL_LOD_FP32_RESCALED;
        so.sampler_precision = o.exact ? SL_SAMPLER_EXACT : SL_SAMPLER_FAST;
        so.lod_flags = SL_LOD_ZERO_OK;
        // the generic L-sampler with its lanes per task chosen by timing (the compact rfunctions made
        // it the faster kernel on the pedigrees measured); with -J, long runs also compile the
        // L-sampler for the pedigree (same draws, same graphs) on a host thread while the run starts
        // on the generic kernel, pedigrees side by side (up to 2000 members: the generated source
        // grows with the peel's shapes, and so does its compile time)
        so.ls_kernel = o.compiled_ls && !o.exact && !o.generic_ls && o.burnin + o.iterations >= 10000 && p.N <= 2000
                           ? SL_LS_KERNEL_BACKGROUND
                           : SL_LS_KERNEL_GENERIC;
        for (int r = 0; r < (o.mc3 ? o.runs : 1) && !rc; ++r) {
            sl_ctx* ctx = nullptr;
            // a fixed scoring kernel keeps the table a function of the seed: the specialised
            // kernel with values in registers, else the slot-program interpreter (the timed
            // choice of SL_LOD_KERNEL_AUTO can differ from run to run in the last FP32 bits)
            if (!o.exact) so.lod_kernel = SL_LOD_KERNEL_JIT_REG;
            if (sl_create(&d, &so, &ctx) != SL_OK && !o.exact) {
                // a kernel compiled at run time did not build: the generic kernels
                fprintf(stderr, "note: pedigree '%s': %s; using the generic kernels\n", fams[f].id.c_str(),
                        sl_last_error(nullptr));
                so.lod_kernel = SL_LOD_KERNEL_INTERP;
                so.ls_kernel = SL_LS_KERNEL_GENERIC;
                ctx = nullptr;
                if (sl_create(&d, &so, &ctx) != SL_OK) ctx = nullptr;
            }
            if (!ctx) {
                fprintf(stderr, "error: pedigree '%s': %s\n", fams[f].id.c_str(), sl_last_error(nullptr));
                rc = 1;
                break;
            }
            const uint64_t si_seed = seed + ctxs.size();
            ctxs.push_back(ctx);
            units.push_back({f, r, ctx});
            if (o.mc3 && sl_set_temperatures(ctx, temps.data()) != SL_OK) {
                fprintf(stderr, "error: pedigree '%s': %s\n", fams[f].id.c_str(), sl_last_error(ctx));
                rc = 1;
                break;
            }
            // sequential imputation (LinkageProgram::run_pedigree): every chain starts from its best pass
            std::vector<double> best(per_ctx);
            if (sl_sequential_imputation_run(ctx, std::max(1, o.si), si_seed, best.data()) != SL_OK) {
                fprintf(stderr, "error: pedigree '%s': %s\n", fams[f].id.c_str(), sl_last_error(ctx));
                rc = 1;
                break;
            }
            if (r == 0)
                fprintf(stderr, "pedigree %s: %d members, starting likelihood (log10) = %.3f\n", fams[f].id.c_str(),
                        p.N, best[0] / std::log(10.0));
        }
    }
    // the MCMC of every pedigree in one batch (with -T: one scoring period at a time, tracing in between)
    if (!rc) {
        sl_batch* b = nullptr;
        if (sl_batch_create(ctxs.data(), (int)ctxs.size(), &b) != SL_OK) {
            fprintf(stderr, "error: %s\n", sl_last_error(nullptr));
            rc = 1;
        } else {
            // trace targets: run r of family f is chain r of the family's context, or chain 0 (t = 1)
            // of its own context under MC3
            struct Trace {
                sl_ctx* ctx;
                int chain;
                FILE* fh;
            };
            std::vector<Trace> traces;
            if (o.trace)
                for (const Unit& u : units)
                    for (int r = 0; r < (o.mc3 ? 1 : o.runs); ++r) {
                        const int run = o.mc3 ? u.run : r;
                        const std::string fn = o.trace_prefix + ".ped" + fams[u.fam].id + ".run" + std::to_string(run);
                        FILE* fh = fopen(fn.c_str(), "w");
                        if (!fh) {
                            fprintf(stderr, "error: could not open trace file '%s'\n", fn.c_str());
                            rc = 1;
                            break;
                        }
                        fprintf(fh, "iteration likelihood\n");
                        fprintf(stderr, "opened trace file (%s)\n", fn.c_str());
                        traces.push_back({u.ctx, o.mc3 ? 0 : r, fh});
                    }
            const int total = o.burnin + o.iterations;
            for (int it = 0, it1; it < total && !rc; it = it1) {
                // iterations [it, it1); with -T a span ends just after a scoring iteration
                // (i >= burnin, i % period == 0), whose trace line is "i+1  log P(G)" (MarkovChain::run,
                // markov_chain.cc:357-370)
                it1 = total;
                if (o.trace) {
                    const int s = std::max(it, o.burnin);
                    it1 = std::min(total, (s + o.period - 1) / o.period * o.period + 1);
                }
                sl_run_options ro{};
                ro.iterations = it1 - o.burnin;
                ro.burnin = o.burnin;
                ro.scoring_period = o.period;
                ro.first_iteration = it;
                ro.lsampler_prob = o.lprob;
                ro.seed = seed;
                ro.exchange_period = o.mc3 && o.chains > 1 ? o.exchange : 0;
                if (it1 <= o.burnin) {
                    ro.iterations = 0;
                    ro.burnin = it1;
                }
                if (sl_batch_run(b, &ro) != SL_OK) {
                    fprintf(stderr, "error: %s\n", sl_last_error(nullptr));
                    rc = 1;
                    break;
                }
                const int last = it1 - 1;
                if (o.trace && last >= o.burnin && last % o.period == 0)
                    for (const Trace& t : traces) {
                        double ll = 0.0;
                        if (sl_chain_loglik(t.ctx, t.chain, t.chain, &ll) != SL_OK) {
                            fprintf(stderr, "error: %s\n", sl_last_error(t.ctx));
                            rc = 1;
                            break;
                        }
                        fprintf(t.fh, "%d\t%f\n", last + 1, ll);
                    }
            }
            for (const Trace& t : traces) fclose(t.fh);
            for (const Unit& u : units) {
                int32_t k = 0;
                double ms = 0.0;
                if (sl_ls_kernel_info(u.ctx, &k, &ms) != SL_OK) continue;
                if (k == SL_LS_KERNEL_GENERIC && ms > 0.0)   // a compile that ended without a kernel
                    fprintf(stderr, "note: pedigree '%s': %s\n", fams[u.fam].id.c_str(), sl_last_error(u.ctx));
                else if (o.verbose && k == SL_LS_KERNEL_SPECIALISED)
                    fprintf(stderr, "pedigree %s run %d: L-sampler compiled for the pedigree in %.1f s\n",
                            fams[u.fam].id.c_str(), u.run, ms / 1000.0);
            }
            if (o.mc3 && o.verbose && !rc)
                for (const Unit& u : units) {
                    std::vector<int64_t> acc(std::max(1, o.chains - 1)), prop(acc.size());
                    if (o.chains > 1 && sl_mc3_stats(u.ctx, acc.data(), prop.data()) == SL_OK)
                        for (int c = 0; c + 1 < o.chains; ++c)
                            fprintf(stderr, "pedigree %s run %d: exchanges %d <-> %d: %lld of %lld accepted\n",
                                    fams[u.fam].id.c_str(), u.run, c, c + 1, (long long)acc[c], (long long)prop[c]);
                }
            sl_batch_destroy(b);
        }
    }
    // LOD table (LinkageWriter::write): per family (raw - log count - P(T)) / log(10), summed; a family's
    // runs in separate contexts are merged first (LODscores::merge_results, lod_score.h:98-105)
    std::vector<std::vector<double>> lod(fams.size(), std::vector<double>((size_t)(M - 1) * n));
    for (size_t f = 0; f < fams.size() && !rc; ++f) {
        std::vector<double> raw, r1((size_t)(M - 1) * n);
        uint64_t count = 0, c1 = 0;
        double tp = 0.0;
        for (const Unit& u : units) {
            if (u.fam != f) continue;
            if (sl_lod_results(u.ctx, r1.data(), &c1, &tp) != SL_OK) {
                fprintf(stderr, "error: pedigree '%s': %s\n", fams[f].id.c_str(), sl_last_error(u.ctx));
                rc = 1;
                break;
            }
            if (raw.empty()) {
                raw = r1;
            } else {
                for (size_t k = 0; k < raw.size(); ++k) raw[k] = log_sum(raw[k], r1[k]);
            }
            count += c1;
        }
        for (size_t k = 0; k < raw.size(); ++k)
            lod[f][k] = (raw[k] - std::log((double)count) - tp) / std::log(10.0);
    }
    if (!rc && !write_table(o, map, partial, lod)) rc = 1;
    for (sl_ctx* c : ctxs) sl_destroy(c);
    return rc;
}
