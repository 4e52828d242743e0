// The adjoint of the trait peel specialised to one pedigree.
//
// trait_adjoint_kernel and trait_adjoint_thr_kernel (sl_kernels.cu) interpret
// per-operation item tables: every (cell, term) item of the dense peel costs
// its table words, a loop over its factors at offsets read from the table,
// the product of the op's recombination terms over the children and a scaling
// of every factor as it is read -- over a hundred instructions per item.  Here
// the same peel (every cell of every rfunction, four terms per cell, the peel
// of TraitRfunction, trait_rfunction.cc:28-137) and its reverse sum-product
// are written out as CUDA C++ for one pedigree and compiled with NVRTC:
//
//  * one forward and one reverse __noinline__ function per operation *shape*
//    (type, cutset size, the positions of the peel node's parents, each
//    previous rfunction's cutset size and key positions, each child's
//    positions), with every cell, term, gather index and transmission mask
//    an immediate; an op's arena offsets, its peel node's disease
//    probabilities and their derivatives, its scaling target and its
//    children's indicator bits are the call's arguments, so ops of one shape
//    share one function (the NVRTC compile and the instruction cache stay
//    small);
//  * one thread per task (graph, interval, position), the task's matrices,
//    adjoints and exponents in a global arena, a 128-float column per block
//    (a thread's float o at o * 128 + threadIdx.x of its block's slice, so
//    the 32 threads of a warp touch one 128-byte line, and every offset is an
//    immediate);
//  * the forward stores each rfunction scaled by a power of two (its largest
//    cell to 2^scale_to, as the other forms do) with its exponent; the reverse
//    of an op reads its cells' adjoints, recomputes its recombination terms
//    and their derivatives by theta_L and theta_R, and writes the adjoints of
//    its previous rfunctions' cells -- each rfunction has one consumer, so
//    every adjoint cell is written once, from registers, with no
//    read-modify-write; the derivatives by the penetrances and the frequency
//    are summed per peel-node state and multiplied by the state's derivative
//    at the end of the op.
//
// The arithmetic is the interpreter's in FP32 (products left to right, the
// four terms of a cell added in order); the reverse sums its contributions
// in a different order, so gradients agree with the other forms to FP32
// rounding, not bit for bit.
#include "sl_adjjit.h"

#include <cuda_runtime.h>

#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "sl_jit.h"

namespace sl {

namespace {

void emitf(std::string& s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void emitf(std::string& s, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    int k = vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (k >= (int)sizeof(buf)) {
        std::vector<char> big(k + 1);
        va_start(ap, fmt);
        vsnprintf(big.data(), big.size(), fmt, ap);
        va_end(ap);
        s.append(big.data(), k);
    } else {
        s.append(buf, k);
    }
}

// The phased trait state of a child whose mother is in state m and father in
// state p, taking the mother's allele i and the father's allele j
// (0 = the first, 1 = the second); states UU, AA, AU, UA (trait.h:21-27).
int phased(int m, int p, int i, int j) {
    const int ma = (m == AA) || (m == AU && i == 0) || (m == UA && i == 1);
    const int pa = (p == AA) || (p == AU && j == 0) || (p == UA && j == 1);
    if (ma) return pa ? (int)AA : (int)AU;
    return pa ? (int)UA : (int)UU;
}

int dig(int ext, int pos) { return (ext >> (2 * pos)) & 3; }

struct Prev {
    int op, c;
    std::vector<int> keys;   // the position of each of its keys in this op's (cutset, peel node) index
};
struct Kid {
    int person, pc, po, mum;
};
struct Shape {
    int type, c, mpos, fpos;
    std::vector<Prev> prev;
    std::vector<Kid> kids;   // CHILD: the peel node; PARENT: its children
};

Shape shape_of(const AdjJitIn& in, int k) {
    const OpDev& op = in.ops[k];
    Shape s;
    s.type = op.type;
    s.c = op.c;
    s.mpos = op.type == CHILD ? op.mpos : -1;
    s.fpos = op.type == CHILD ? op.fpos : -1;
    const int32_t* pd = in.od + op.prev_at;
    const int32_t* po = in.od + op.prev_ops_at;
    for (int j = 0; j < op.n_prev; ++j) {
        Prev p;
        p.op = po[j];
        p.c = pd[1];
        p.keys.assign(pd + 2, pd + 2 + pd[1]);
        s.prev.push_back(p);
        pd += 2 + pd[1];
    }
    if (op.type == CHILD) s.kids.push_back(Kid{op.peel, -1, -1, 0});
    if (op.type == PARENT)
        for (int c = 0; c < op.n_child; ++c) {
            const int32_t* cd = in.od + op.child_at + 4 * c;
            s.kids.push_back(Kid{cd[0], cd[1], cd[2], cd[3]});
        }
    return s;
}

std::string shape_key(const Shape& s) {
    std::string k;
    emitf(k, "%d %d %d %d |", s.type, s.c, s.mpos, s.fpos);
    for (const Prev& p : s.prev) {
        emitf(k, " %d:", p.c);
        for (int q : p.keys) emitf(k, "%d,", q);
    }
    k += " |";
    if (s.type == PARENT)
        for (const Kid& c : s.kids) emitf(k, " %d,%d,%d", c.pc, c.po, c.mum);
    return k;
}

// One (cell, term) item of the dense peel: the peel node's state, the cell of
// every previous rfunction it gathers, and for a parent peel the mask of each
// child's transmissions (i, j) -> bit 2i + j that give the child's state.
struct Item {
    int s;
    std::vector<int> idx;
    std::vector<int> mask;
    bool zero;   // a child's state is unreachable: the term is exactly zero
};

std::vector<Item> items_of(const Shape& sh) {
    std::vector<Item> out;
    const int ncell = 1 << (2 * sh.c);
    for (int cell = 0; cell < ncell; ++cell)
        for (int t = 0; t < 4; ++t) {
            Item it;
            it.zero = false;
            it.s = sh.type == CHILD ? phased(dig(cell, sh.mpos), dig(cell, sh.fpos), t >> 1, t & 1) : t;
            const int ext = cell | (it.s << (2 * sh.c));
            for (const Prev& p : sh.prev) {
                int idx = 0;
                for (size_t q = 0; q < p.keys.size(); ++q) idx |= dig(ext, p.keys[q]) << (2 * q);
                it.idx.push_back(idx);
            }
            if (sh.type == PARENT) {
                int mt = t, pt = t;
                for (const Kid& c : sh.kids) {
                    const int kt = dig(ext, c.pc), other = dig(ext, c.po);
                    if (c.mum) pt = other; else mt = other;
                    int mask = 0;
                    for (int i = 0; i < 2; ++i)
                        for (int j = 0; j < 2; ++j)
                            if (phased(mt, pt, i, j) == kt) mask |= 1 << (2 * i + j);
                    it.mask.push_back(mask);
                    if (!mask) it.zero = true;
                }
            }
            out.push_back(it);
        }
    return out;
}

std::string func_params(const Shape& sh, bool reverse) {
    std::string s = "float* __restrict__ Ab, int oK, int eK";
    for (size_t j = 0; j < sh.prev.size(); ++j) emitf(s, ", int o%zu", j);
    s += ", const float* __restrict__ dp";
    if (reverse) s += ", const float4* __restrict__ dg";
    else s += ", int sct";
    for (size_t c = 0; c < sh.kids.size(); ++c) emitf(s, ", u32 wl%zu, u32 wr%zu, int bt%zu", c, c, c);
    s += ", float th, float an, float th2, float an2";
    return s;
}

// 0.25 x the recombination term (i, j) of kid c and, for the reverse, its
// derivatives by theta_L and theta_R (TraitRfunction::get_recombination_probability,
// trait_rfunction.cc:9-24): x0 the maternal allele at the left marker, x1 at
// the right, x2 and x3 the paternal ones.
void emit_rec(std::string& s, size_t c, bool deriv) {
    emitf(s,
          "    const bool ml%zu = (wl%zu >> bt%zu) & 1u, pl%zu = (wl%zu >> (bt%zu + 1)) & 1u, mr%zu = (wr%zu >> bt%zu) & 1u, "
          "pr%zu = (wr%zu >> (bt%zu + 1)) & 1u;\n",
          c, c, c, c, c, c, c, c, c, c, c, c);
    for (int b = 0; b < 4; ++b) {
        const int i = b >> 1, j = b & 1;
        const char* eqi = i ? "" : "!";
        const char* eqj = j ? "" : "!";
        emitf(s,
              "    const float x0_%zu_%d = %sml%zu ? an : th, x1_%zu_%d = %smr%zu ? an2 : th2, x2_%zu_%d = %spl%zu ? an : th, "
              "x3_%zu_%d = %spr%zu ? an2 : th2;\n",
              c, b, eqi, c, c, b, eqi, c, c, b, eqj, c, c, b, eqj, c);
        emitf(s, "    const float r%zu_%d = 0.25f * (((x0_%zu_%d * x1_%zu_%d) * x2_%zu_%d) * x3_%zu_%d);\n", c, b, c, b, c,
              b, c, b, c, b);
        if (deriv) {
            emitf(s,
                  "    const float s0_%zu_%d = %sml%zu ? -1.0f : 1.0f, s1_%zu_%d = %smr%zu ? -1.0f : 1.0f, s2_%zu_%d = "
                  "%spl%zu ? -1.0f : 1.0f, s3_%zu_%d = %spr%zu ? -1.0f : 1.0f;\n",
                  c, b, eqi, c, c, b, eqi, c, c, b, eqj, c, c, b, eqj, c);
            emitf(s,
                  "    const float dl%zu_%d = 0.25f * (((s0_%zu_%d * x1_%zu_%d) * x2_%zu_%d) * x3_%zu_%d + "
                  "((x0_%zu_%d * x1_%zu_%d) * s2_%zu_%d) * x3_%zu_%d);\n",
                  c, b, c, b, c, b, c, b, c, b, c, b, c, b, c, b, c, b);
            emitf(s,
                  "    const float dr%zu_%d = 0.25f * (((x0_%zu_%d * s1_%zu_%d) * x2_%zu_%d) * x3_%zu_%d + "
                  "((x0_%zu_%d * x1_%zu_%d) * x2_%zu_%d) * s3_%zu_%d);\n",
                  c, b, c, b, c, b, c, b, c, b, c, b, c, b, c, b, c, b);
        }
    }
}

// The recombination factor of an item (and its derivatives): a child peel's
// term r[t]; a parent peel's product over children of the sum of the
// transmissions its mask lets through (adj_R in sl_kernels.cu), memoised per
// mask tuple.  Returns the names of (R, dRl, dRr); "" for R = 1.
struct RecNames {
    std::string R, dl, dr;
};

class RecEmitter {
  public:
    RecEmitter(std::string& s, const Shape& sh, bool deriv) : s_(s), sh_(sh), deriv_(deriv) {}
    RecNames get(const Item& it, int t) {
        if (sh_.type == CHILD) {
            char b[3][32];
            snprintf(b[0], 32, "r0_%d", t);
            snprintf(b[1], 32, "dl0_%d", t);
            snprintf(b[2], 32, "dr0_%d", t);
            return RecNames{b[0], b[1], b[2]};
        }
        if (sh_.type != PARENT) return RecNames{"", "", ""};
        auto f = memo_.find(it.mask);
        if (f != memo_.end()) return f->second;
        // per-child sums
        std::vector<std::string> S, Sl, Sr;
        for (size_t c = 0; c < it.mask.size(); ++c) {
            const int m = it.mask[c];
            const auto key = std::make_pair((int)c, m);
            if (!sums_.count(key)) {
                std::string e, el, er;
                for (int b = 0; b < 4; ++b)
                    if (m & (1 << b)) {
                        char x[32];
                        snprintf(x, sizeof x, "r%zu_%d", c, b);
                        e = e.empty() ? std::string(x) : "(" + e + " + " + x + ")";
                        if (deriv_) {
                            snprintf(x, sizeof x, "dl%zu_%d", c, b);
                            el = el.empty() ? std::string(x) : "(" + el + " + " + x + ")";
                            snprintf(x, sizeof x, "dr%zu_%d", c, b);
                            er = er.empty() ? std::string(x) : "(" + er + " + " + x + ")";
                        }
                    }
                emitf(s_, "    const float S%zu_%d = %s;\n", c, m, e.c_str());
                if (deriv_) emitf(s_, "    const float Sl%zu_%d = %s, Sr%zu_%d = %s;\n", c, m, el.c_str(), c, m, er.c_str());
                sums_.insert(key);
            }
            char x[32];
            snprintf(x, sizeof x, "S%zu_%d", c, m);
            S.push_back(x);
            snprintf(x, sizeof x, "Sl%zu_%d", c, m);
            Sl.push_back(x);
            snprintf(x, sizeof x, "Sr%zu_%d", c, m);
            Sr.push_back(x);
        }
        const int id = (int)memo_.size();
        RecNames rn;
        char nm[32];
        snprintf(nm, sizeof nm, "R%d", id);
        rn.R = nm;
        snprintf(nm, sizeof nm, "Rl%d", id);
        rn.dl = nm;
        snprintf(nm, sizeof nm, "Rr%d", id);
        rn.dr = nm;
        // the product rule in child order: dR = dR * S_c + R * dS_c, R *= S_c
        std::string R = S[0], dl = Sl[0], dr = Sr[0];
        for (size_t c = 1; c < S.size(); ++c) {
            if (deriv_) {
                dl = "(" + dl + " * " + S[c] + " + " + R + " * " + Sl[c] + ")";
                dr = "(" + dr + " * " + S[c] + " + " + R + " * " + Sr[c] + ")";
            }
            R = "(" + R + " * " + S[c] + ")";
        }
        emitf(s_, "    const float %s = %s;\n", rn.R.c_str(), R.c_str());
        if (deriv_) emitf(s_, "    const float %s = %s, %s = %s;\n", rn.dl.c_str(), dl.c_str(), rn.dr.c_str(), dr.c_str());
        memo_[it.mask] = rn;
        return rn;
    }

  private:
    std::string& s_;
    const Shape& sh_;
    bool deriv_;
    std::map<std::vector<int>, RecNames> memo_;
    std::set<std::pair<int, int>> sums_;
};

// A previous rfunction's cell as a register, loaded at first use.
class PrevLoads {
  public:
    explicit PrevLoads(std::string& s) : s_(s) {}
    std::string get(size_t j, int idx) {
        const auto key = std::make_pair((int)j, idx);
        char nm[32];
        snprintf(nm, sizeof nm, "a%zu_%d", j, idx);
        if (!seen_.count(key)) {
            emitf(s_, "    const float %s = p%zu[%d];\n", nm, j, idx * kAdjJitThreads);
            seen_.insert(key);
        }
        return nm;
    }

  private:
    std::string& s_;
    std::set<std::pair<int, int>> seen_;
};

// 2^-e as a multiplier when it is a normal number, else 0 (then ldexpf).
const char* kPow2 =
    "__device__ __forceinline__ float pw2n(int e) {\n"
    "  return (e >= -127 && e <= 126) ? __int_as_float((127 - e) << 23) : 0.0f;\n"
    "}\n";

void emit_forward(std::string& s, const Shape& sh, int id) {
    const std::vector<Item> items = items_of(sh);
    const int ncell = 1 << (2 * sh.c);
    emitf(s, "__device__ __noinline__ void F%d(%s) {\n", id, func_params(sh, false).c_str());
    s += "    const float d0 = dp[0], d1 = dp[1], d2 = dp[2], d3 = dp[3];\n";
    s += "    float* o = Ab + oK;\n";
    for (size_t j = 0; j < sh.prev.size(); ++j) emitf(s, "    const float* p%zu = Ab + o%zu;\n", j, j);
    if (sh.type == CHILD || sh.type == PARENT)
        for (size_t c = 0; c < sh.kids.size(); ++c) emit_rec(s, c, false);
    RecEmitter rec(s, sh, false);
    PrevLoads pl(s);
    for (int cell = 0; cell < ncell; ++cell) {
        std::string sum;
        for (int t = 0; t < 4; ++t) {
            const Item& it = items[4 * cell + t];
            if (it.zero) continue;
            std::string term = "d" + std::to_string(it.s);
            for (size_t j = 0; j < sh.prev.size(); ++j) term = "(" + term + " * " + pl.get(j, it.idx[j]) + ")";
            const RecNames rn = rec.get(it, t);
            if (!rn.R.empty()) term = "(" + term + " * " + rn.R + ")";
            sum = sum.empty() ? term : "(" + sum + " + " + term + ")";
        }
        if (sum.empty()) sum = "0.0f";
        emitf(s, "    const float u%d = %s;\n", cell, sum.c_str());
    }
    s += "    float mx = 0.0f;\n";
    for (int cell = 0; cell < ncell; ++cell) emitf(s, "    mx = fmaxf(mx, u%d);\n", cell);
    s += "    const int e = mx > 0.0f ? ilogbf(mx) - sct : 0;\n";
    s += "    const float sc = pw2n(e);\n";
    s += "    reinterpret_cast<int*>(Ab)[eK] = e;\n";
    s += "    if (sc != 0.0f) {\n";
    for (int cell = 0; cell < ncell; ++cell) emitf(s, "        o[%d] = u%d * sc;\n", cell * kAdjJitThreads, cell);
    s += "    } else {\n";
    for (int cell = 0; cell < ncell; ++cell) emitf(s, "        o[%d] = ldexpf(u%d, -e);\n", cell * kAdjJitThreads, cell);
    s += "    }\n}\n";
}

void emit_reverse(std::string& out, const Shape& sh, int id) {
    const std::vector<Item> items = items_of(sh);
    const int ncell = 1 << (2 * sh.c);
    const bool hasR = sh.type == CHILD || sh.type == PARENT;
    emitf(out, "__device__ __noinline__ G6 R%d(%s) {\n", id, func_params(sh, true).c_str());
    std::string s;   // the body; the adjoint registers' declarations go before it
    s += "    const float d0 = dp[0], d1 = dp[1], d2 = dp[2], d3 = dp[3];\n";
    s += "    const float* bk = Ab + HB + oK;\n";
    for (size_t j = 0; j < sh.prev.size(); ++j)
        emitf(s, "    const float* p%zu = Ab + o%zu;\n    float* q%zu = Ab + HB + o%zu;\n", j, j, j, j);
    // the cells' adjoints before their scaling
    s += "    const int e = reinterpret_cast<const int*>(Ab)[eK];\n";
    s += "    const float sk = pw2n(e);\n";
    for (int cell = 0; cell < ncell; ++cell) emitf(s, "    const float b%d = bk[%d];\n", cell, cell * kAdjJitThreads);
    emitf(s, "    float gd[%d];\n", ncell);
    s += "    if (sk != 0.0f) {\n";
    for (int cell = 0; cell < ncell; ++cell) emitf(s, "        gd[%d] = b%d * sk;\n", cell, cell);
    s += "    } else {\n";
    for (int cell = 0; cell < ncell; ++cell) emitf(s, "        gd[%d] = ldexpf(b%d, -e);\n", cell, cell);
    s += "    }\n";
    if (hasR)
        for (size_t c = 0; c < sh.kids.size(); ++c) emit_rec(s, c, true);
    s += "    float gs0 = 0.0f, gs1 = 0.0f, gs2 = 0.0f, gs3 = 0.0f;\n";
    if (hasR) s += "    float ls0 = 0.0f, ls1 = 0.0f, ls2 = 0.0f, ls3 = 0.0f, rs0 = 0.0f, rs1 = 0.0f, rs2 = 0.0f, rs3 = 0.0f;\n";
    RecEmitter rec(s, sh, true);
    PrevLoads pl(s);
    std::map<std::pair<int, int>, bool> started;   // (prev, cell) -> its adjoint register exists
    const size_t np = sh.prev.size();
    for (int cell = 0; cell < ncell; ++cell)
        for (int t = 0; t < 4; ++t) {
            const Item& it = items[4 * cell + t];
            if (it.zero) continue;
            std::vector<std::string> a(np);
            for (size_t j = 0; j < np; ++j) a[j] = pl.get(j, it.idx[j]);
            const RecNames rn = rec.get(it, t);
            std::string pp;
            for (size_t j = 0; j < np; ++j) pp = pp.empty() ? a[j] : "(" + pp + " * " + a[j] + ")";
            const std::string wgt = pp.empty() ? "gd[" + std::to_string(cell) + "]"
                                               : "(gd[" + std::to_string(cell) + "] * " + pp + ")";
            emitf(s, "    { const float w = %s;\n", wgt.c_str());
            if (hasR) {
                emitf(s, "      gs%d += w * %s; ls%d += w * %s; rs%d += w * %s;\n", it.s, rn.R.c_str(), it.s,
                      rn.dl.c_str(), it.s, rn.dr.c_str());
            } else {
                emitf(s, "      gs%d += w;\n", it.s);
            }
            if (np > 0) {
                std::string run = "(gd[" + std::to_string(cell) + "] * d" + std::to_string(it.s) + ")";
                if (hasR) run = "(" + run + " * " + rn.R + ")";
                emitf(s, "      const float run = %s;\n", run.c_str());
                // each factor's adjoint: the product of the others, prefix then suffix
                std::vector<std::string> pre(np);
                std::string p = "run";
                for (size_t j = 0; j < np; ++j) {
                    pre[j] = p;
                    p = "(" + p + " * " + a[j] + ")";
                }
                std::string suf;
                for (size_t jj = np; jj-- > 0;) {
                    const std::string v = suf.empty() ? pre[jj] : "(" + pre[jj] + " * " + suf + ")";
                    const auto key = std::make_pair((int)jj, it.idx[jj]);
                    if (!started.count(key)) {
                        started[key] = true;
                        emitf(s, "      g%zu_%d = %s;\n", jj, it.idx[jj], v.c_str());
                    } else {
                        emitf(s, "      g%zu_%d += %s;\n", jj, it.idx[jj], v.c_str());
                    }
                    suf = suf.empty() ? a[jj] : "(" + suf + " * " + a[jj] + ")";
                }
            }
            s += "    }\n";
        }
    for (size_t j = 0; j < np; ++j) {
        const int n = 1 << (2 * sh.prev[j].c);
        for (int idx = 0; idx < n; ++idx)
            if (started.count(std::make_pair((int)j, idx))) emitf(out, "    float g%zu_%d;\n", j, idx);
    }
    for (size_t j = 0; j < np; ++j) {
        const int n = 1 << (2 * sh.prev[j].c);
        for (int idx = 0; idx < n; ++idx) {
            if (started.count(std::make_pair((int)j, idx)))
                emitf(s, "    q%zu[%d] = g%zu_%d;\n", j, idx * kAdjJitThreads, j, idx);
            else
                emitf(s, "    q%zu[%d] = 0.0f;\n", j, idx * kAdjJitThreads);
        }
    }
    s += "    const float4 c0 = dg[0], c1 = dg[1], c2 = dg[2], c3 = dg[3];\n";
    s += "    G6 g;\n";
    if (hasR) {
        s += "    g.l = ((d0 * ls0 + d1 * ls1) + d2 * ls2) + d3 * ls3;\n";
        s += "    g.r = ((d0 * rs0 + d1 * rs1) + d2 * rs2) + d3 * rs3;\n";
    } else {
        s += "    g.l = 0.0f;\n    g.r = 0.0f;\n";
    }
    s += "    g.p0 = ((gs0 * c0.x + gs1 * c1.x) + gs2 * c2.x) + gs3 * c3.x;\n";
    s += "    g.p1 = ((gs0 * c0.y + gs1 * c1.y) + gs2 * c2.y) + gs3 * c3.y;\n";
    s += "    g.p2 = ((gs0 * c0.z + gs1 * c1.z) + gs2 * c2.z) + gs3 * c3.z;\n";
    s += "    g.q = ((gs0 * c0.w + gs1 * c1.w) + gs2 * c2.w) + gs3 * c3.w;\n";
    s += "    return g;\n}\n";
    out += s;
}

}  // namespace

std::string adj_jit_source(const AdjJitIn& in, int* shapes_out, int* half_out) {
    const int K = in.K;
    std::vector<int> aoff(K);
    int half = 0;
    for (int k = 0; k < K; ++k) {
        aoff[k] = half;
        half += 1 << (2 * in.ops[k].c);
    }
    std::map<std::string, int> shape_id;
    std::vector<Shape> shapes(K);
    std::vector<int> sid(K);
    std::vector<Shape> uniq;
    for (int k = 0; k < K; ++k) {
        shapes[k] = shape_of(in, k);
        const std::string key = shape_key(shapes[k]);
        auto it = shape_id.find(key);
        if (it == shape_id.end()) {
            const int id = (int)uniq.size();
            shape_id[key] = id;
            uniq.push_back(shapes[k]);
            sid[k] = id;
        } else {
            sid[k] = it->second;
        }
    }
    const int64_t npos = (int64_t)(in.M - 1) * in.n;
    std::string s;
    s.reserve(1 << 20);
    s += "typedef unsigned int u32;\n";
    emitf(s, "#define HB %lld\n", (long long)half * kAdjJitThreads);
    s += "struct G6 { float l, r, p0, p1, p2, q; };\n";
    s += kPow2;
    for (size_t i = 0; i < uniq.size(); ++i) {
        emit_forward(s, uniq[i], (int)i);
        emit_reverse(s, uniq[i], (int)i);
    }
    // the kernel: one thread per task, a persistent grid over the tasks
    std::set<int> kids;
    for (int k = 0; k < K; ++k)
        for (const Kid& c : shapes[k].kids) kids.insert(c.person);
    std::set<int> words;
    for (int p : kids) words.insert((2 * (p - in.F)) >> 5);
    emitf(s,
          "extern \"C\" __global__ void __launch_bounds__(%d, %d) sl_adj_jit(const u32* __restrict__ graphs, long long gw,\n"
          "    long long task0, long long ntask, double* __restrict__ grad, int* status,\n"
          "    const float* __restrict__ partial, float* __restrict__ arena, const float* __restrict__ dprob,\n"
          "    const float4* __restrict__ dgrad, int zero_ok) {\n",
          kAdjJitThreads, in.min_blocks > 0 ? in.min_blocks : 1);
    emitf(s, "  float* Ab = arena + (long long)blockIdx.x * %lldLL + threadIdx.x;\n",
          (long long)adj_jit_block_floats(half, K));
    emitf(s, "  const long long npos = %lldLL;\n", (long long)npos);
    emitf(s, "  for (long long u = (long long)blockIdx.x * %d + threadIdx.x; u < ntask; u += (long long)gridDim.x * %d) {\n",
          kAdjJitThreads, kAdjJitThreads);
    s += "    const long long t = task0 + u;\n";
    s += "    const int b = (int)(t / npos);\n    const int pidx = (int)(t % npos);\n";
    emitf(s, "    const int l = pidx / %d, o = pidx %% %d;\n", in.n, in.n);
    emitf(s, "    const u32* cL = graphs + (long long)b * gw + (long long)l * %d;\n    const u32* cR = cL + %d;\n", in.W,
          in.W);
    for (int w : words) emitf(s, "    const u32 wL%d = cL[%d], wR%d = cR[%d];\n", w, w, w, w);
    emitf(s, "    const float th = partial[l] * (float)(o + 1), th2 = partial[l] * (float)(%d - o);\n", in.n);
    s += "    const float an = 1.0f - th, an2 = 1.0f - th2;\n";
    auto args = [&](int k, bool reverse) {
        const OpDev& op = in.ops[k];
        std::string a;
        emitf(a, "Ab, %d, %lld", aoff[k] * kAdjJitThreads, (long long)(2 * half + k) * kAdjJitThreads);
        for (const Prev& p : shapes[k].prev) emitf(a, ", %d", aoff[p.op] * kAdjJitThreads);
        emitf(a, ", dprob + %d", 4 * op.peel);
        if (reverse) emitf(a, ", dgrad + %d", 4 * op.peel);
        else emitf(a, ", %d", op.scale_to);
        for (const Kid& c : shapes[k].kids) {
            // the kid's indicator bits (maternal, paternal) at both markers: word, and bit of the maternal one
            const int bpos = 2 * (c.person - in.F);
            emitf(a, ", wL%d, wR%d, %d", bpos >> 5, bpos >> 5, bpos & 31);
        }
        a += ", th, an, th2, an2";
        return a;
    };
    for (int k = 0; k < K; ++k) emitf(s, "    F%d(%s);\n", sid[k], args(k, false).c_str());
    emitf(s, "    const float root = Ab[%d];\n", aoff[K - 1] * kAdjJitThreads);
    emitf(s,
          "    if (!(root > 0.0f)) {\n"
          "      if (!zero_ok) atomicCAS(status, 0, %d);\n"
          "      for (int q = 0; q < 6; ++q) grad[u * 6 + q] = __longlong_as_double(0x7ff8000000000000LL);\n"
          "      continue;\n    }\n",
          (int)ST_LOD_NONPOS);
    emitf(s, "    Ab[HB + %d] = 1.0f / root;\n", aoff[K - 1] * kAdjJitThreads);
    s += "    double g0 = 0.0, g1 = 0.0, g2 = 0.0, g3 = 0.0, g4 = 0.0, g5 = 0.0;\n";
    for (int k = K - 1; k >= 0; --k) {
        emitf(s,
              "    { const G6 r = R%d(%s); g0 += (double)r.l; g1 += (double)r.r; g2 += (double)r.p0; g3 += (double)r.p1; "
              "g4 += (double)r.p2; g5 += (double)r.q; }\n",
              sid[k], args(k, true).c_str());
    }
    s += "    double* gp = grad + u * 6;\n";
    s += "    gp[0] = g0; gp[1] = g1; gp[2] = g2; gp[3] = g3; gp[4] = g4; gp[5] = g5;\n";
    s += "  }\n}\n";
    if (shapes_out) *shapes_out = (int)uniq.size();
    if (half_out) *half_out = half;
    return s;
}

int adj_jit_compile(const AdjJitIn& in, AdjJit* out, std::string* log) {
    *out = AdjJit{};
    const auto t0 = std::chrono::steady_clock::now();
    int shapes = 0, half = 0;
    const std::string src = adj_jit_source(in, &shapes, &half);
    if (jit_compile_kernel(src, "sl_adj_jit.cu", "sl_adj_jit", &out->lib, &out->kern, log)) return -1;
    out->half = half;
    out->shapes = shapes;
    out->min_blocks = in.min_blocks;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, (const void*)out->kern) == cudaSuccess) {
        out->regs = fa.numRegs;
        out->local_bytes = (int)fa.localSizeBytes;
    }
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, (const void*)out->kern, kAdjJitThreads, 0) !=
            cudaSuccess ||
        blocks < 1) {
        adj_jit_release(out);
        *log = "specialised adjoint kernel cannot be resident";
        return -1;
    }
    out->blocks_per_sm = blocks;
    out->compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

void adj_jit_release(AdjJit* j) {
    if (j && j->lib) cudaLibraryUnload((cudaLibrary_t)j->lib);
    if (j) *j = AdjJit{};
}

cudaError_t adj_jit_launch(const AdjJit& j, const uint32_t* graphs, int64_t graph_words, int64_t task0,
                           int64_t ntask, double* grad, int* status, const float* partial, float* arena,
                           int64_t blocks, const float* dprob, const float4* dgrad, int zero_ok, cudaStream_t s) {
    int64_t grid = (ntask + kAdjJitThreads - 1) / kAdjJitThreads;
    if (grid > blocks) grid = blocks;
    if (grid < 1) grid = 1;
    long long gw = graph_words, t0 = task0, nt = ntask;
    void* args[] = {(void*)&graphs, (void*)&gw, (void*)&t0, (void*)&nt, (void*)&grad, (void*)&status,
                    (void*)&partial, (void*)&arena, (void*)&dprob, (void*)&dgrad, (void*)&zero_ok};
    return cudaLaunchKernel((const void*)j.kern, dim3((unsigned)grid), dim3(kAdjJitThreads), args, 0, s);
}

}  // namespace sl
