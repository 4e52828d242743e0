// The FP32 L-sampler specialised to one pedigree: CUDA C++ generated at
// context creation from the peel operations and compiled with NVRTC.
//
// It performs the same steps, in the same rounded operations and order
// (intrinsics that are never contracted, as Ls<float> uses), as ls_locus<float>
// in sl_kernels.cu (LocusSampler::step, locus_sampler2.cc:128-159; the forward
// peel of SamplerRfunction::evaluate, sampler_rfunction.cc:102-287, and the
// backward sampling of SamplerRfunction::sample, sampler_rfunction.cc:
// 290-419): one warp per (chain, locus), one (cell, state) term per lane in
// the forward peel, every rfunction rescaled by a power of two, lane 0 drawing
// each peeled member's ordered genotype, then the meiosis indicators by
// ballot.  What the interpreter reads from the operation lists at run time
// (cutset members, the previous rfunctions' offsets and key positions, the
// children and their parents' positions) is written into the code as
// constants, so a term is a short chain of shared-memory loads and products.
#include "sl_lsjit.h"

#include <cstdarg>
#include <chrono>
#include <memory>
#include <string>
#include <vector>

#include "sl_internal.h"
#include "sl_jit.h"

namespace sl {

namespace {

const char* kPhiloxSrc =
#include "sl_philox_src.inc"
    ;

void emitf(std::string& s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void emitf(std::string& s, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    const int n = vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (n < (int)sizeof buf) {
        s += buf;
        return;
    }
    std::string big((size_t)n + 1, '\0');
    va_start(ap, fmt);
    vsnprintf(&big[0], big.size(), fmt, ap);
    va_end(ap);
    big.resize((size_t)n);
    s += big;
}

size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// Per-warp shared layout, as ls_warp_bytes<float> but without the block's
// operation tables (they are constants here).
struct Layout {
    size_t dist, assign, draws, gcol, cols, pri, total;
};

Layout layout(const JitLsIn& in) {
    Layout L;
    L.dist = (size_t)in.arena * 4;
    L.assign = L.dist + (size_t)in.max_child * 16 * 4;
    L.draws = al16(L.assign + (size_t)in.N);
    L.gcol = al16(L.draws + 8 * (size_t)in.K);
    L.cols = al16(L.gcol + (size_t)in.N);
    L.pri = al16(L.cols + 8 * (size_t)in.W);
    L.total = al16(L.pri + 16 * 4);
    return L;
}

// digit q of the extended cell index (cutset digits, then the peel node's state)
std::string dig(const char* var, int pos) {
    char b[64];
    snprintf(b, sizeof b, "((%s >> %d) & 3)", var, 2 * pos);
    return b;
}

// Operations of the same shape (type, cutset size, the positions the terms
// read, the children's structure) share one generated function; what differs
// between them (the peel node, the cutset members, the rfunction offsets, the
// children's meiosis bits) is passed in.  Fewer, reused functions compile
// faster and keep the instruction footprint small.
struct Shape {
    std::string key;
    int type, c, mpos, fpos, n_prev, n_child;
    std::vector<std::vector<int>> prev_pos;   // per previous rfunction: its keys' positions
    std::vector<int> cpos, opos, pim;         // per child: its position, the other parent's, peel is mother
};

Shape shape_of(const JitLsIn& in, const OpDev& op) {
    Shape sh;
    sh.type = op.type;
    sh.c = op.c;
    sh.mpos = op.type == CHILD ? op.mpos : -1;
    sh.fpos = op.type == CHILD ? op.fpos : -1;
    sh.n_prev = op.n_prev;
    sh.n_child = op.type == PARENT ? op.n_child : 0;
    std::string k = std::to_string(sh.type) + "|" + std::to_string(sh.c) + "|" + std::to_string(sh.mpos) + "," +
                    std::to_string(sh.fpos) + "|";
    const int32_t* pd = in.opdata + op.prev_at;
    for (int j = 0; j < op.n_prev; ++j) {
        const int pc = pd[1];
        std::vector<int> pos(pd + 2, pd + 2 + pc);
        k += "p";
        for (int x : pos) k += std::to_string(x) + ".";
        sh.prev_pos.push_back(pos);
        pd += 2 + pc;
    }
    k += "|";
    const int32_t* cd = in.opdata + op.child_at;
    for (int c = 0; c < sh.n_child; ++c, cd += 4) {
        sh.cpos.push_back(cd[1]);
        sh.opos.push_back(cd[2]);
        sh.pim.push_back(cd[3]);
        k += "c" + std::to_string(cd[1]) + "." + std::to_string(cd[2]) + "." + std::to_string(cd[3]);
    }
    sh.key = k;
    return sh;
}

// An operation's values that a shape function takes as parameters: the peel
// node, its rfunction's offset, the cutset members, the previous rfunctions'
// offsets, the children's (or the peeled child's) first meiosis bits.
std::vector<std::string> value_names(const Shape& sh) {
    std::vector<std::string> n = {"pe", "mat"};
    for (int q = 0; q < sh.c; ++q) n.push_back("cu" + std::to_string(q));
    for (int j = 0; j < sh.n_prev; ++j) n.push_back("mo" + std::to_string(j));
    if (sh.type == CHILD) n.push_back("cb0");
    for (int c = 0; c < sh.n_child; ++c) n.push_back("cb" + std::to_string(c));
    return n;
}

std::vector<int> op_values(const JitLsIn& in, const OpDev& op) {
    std::vector<int> v = {op.peel, op.mat_off};
    const int32_t* cut = in.opdata + op.cut_at;
    for (int q = 0; q < op.c; ++q) v.push_back(cut[q]);
    const int32_t* pd = in.opdata + op.prev_at;
    for (int j = 0; j < op.n_prev; ++j) {
        v.push_back(pd[0]);
        pd += 2 + pd[1];
    }
    if (op.type == CHILD) v.push_back(2 * (op.peel - in.F));
    if (op.type == PARENT) {
        const int32_t* cd = in.opdata + op.child_at;
        for (int c = 0; c < op.n_child; ++c) v.push_back(2 * (cd[4 * c] - in.F));
    }
    return v;
}

std::string call_args(const JitLsIn& in, const OpDev& op) {
    std::string a;
    for (int x : op_values(in, op)) a += (a.empty() ? "" : ", ") + std::to_string(x);
    return a;
}

// the same values as constants, for a function made for one operation
std::string const_prologue(const JitLsIn& in, const OpDev& op, const Shape& sh) {
    const std::vector<std::string> n = value_names(sh);
    const std::vector<int> v = op_values(in, op);
    std::string out = "  const int ";
    for (size_t i = 0; i < n.size(); ++i) out += (i ? ", " : "") + n[i] + " = " + std::to_string(v[i]);
    return out + ";\n";
}

std::string params(const Shape& sh) {
    std::string p;
    for (const std::string& x : value_names(sh)) p += (p.empty() ? "int " : ", int ") + x;
    return p;
}

// The product of one (cell, state) presum entry: tv times the child's
// transmission, the previous rfunctions in order, the children's
// transmissions (ls_term in sl_kernels.cu).
void emit_term(std::string& s, const Shape& sh, const char* ind) {
    emitf(s, "%sfloat tmp = tv;\n", ind);
    if (sh.type == CHILD)
        emitf(s, "%stmp = __fmul_rn(tmp, __fmul_rn(dist[%s * 2 + matA(v)], dist[8 + %s * 2 + patA(v)]));\n", ind,
              dig("ext", sh.mpos).c_str(), dig("ext", sh.fpos).c_str());
    for (int j = 0; j < sh.n_prev; ++j) {
        std::string idx;
        for (size_t q = 0; q < sh.prev_pos[j].size(); ++q) {
            if (q) idx += " | ";
            char b[96];
            snprintf(b, sizeof b, "(%s << %d)", dig("ext", sh.prev_pos[j][q]).c_str(), 2 * (int)q);
            idx += b;
        }
        if (idx.empty()) idx = "0";
        emitf(s, "%stmp = __fmul_rn(tmp, A[mo%d + (%s)]);\n", ind, j, idx.c_str());
    }
    if (sh.type == PARENT) {
        emitf(s, "%s{\n%s  float cp = 1.0f;\n", ind, ind);
        for (int c = 0; c < sh.n_child; ++c) {
            const std::string kt = dig("ext", sh.cpos[c]), ot = dig("ext", sh.opos[c]);
            const std::string mt = sh.pim[c] ? "v" : ot, pt = sh.pim[c] ? ot : "v";
            emitf(s, "%s  { const int kt = %s; cp = __fmul_rn(cp, __fmul_rn(dist[%d + (%s) * 2 + matA(kt)], dist[%d + (%s) * 2 + patA(kt)])); }\n",
                  ind, kt.c_str(), 16 * c, mt.c_str(), 16 * c + 8, pt.c_str());
        }
        emitf(s, "%s  tmp = __fmul_rn(tmp, cp);\n%s}\n", ind, ind);
    }
}

// the validity of a cutset index under the members' genotype-elimination masks
std::string valid_expr(const Shape& sh, const char* var) {
    std::string e;
    for (int q = 0; q < sh.c; ++q) {
        char b[96];
        snprintf(b, sizeof b, "%s((g%d >> ((%s >> %d) & 3)) & 1)", q ? " && " : "", q, var, 2 * q);
        e += b;
    }
    return e.empty() ? std::string("true") : e;
}

void emit_dists(std::string& s, const Shape& sh) {
    if (sh.type == CHILD) {
        s += "      if (lane == 0) dist_one(cb0, cL, cR, th, an, th2, an2, dist);\n";
    } else if (sh.n_child > 0) {
        s += "      if (lane < " + std::to_string(sh.n_child) + ") {\n        int b = 0;\n";
        for (int c = 0; c < sh.n_child; ++c) emitf(s, "        if (lane == %d) b = cb%d;\n", c, c);
        s += "        dist_one(b, cL, cR, th, an, th2, an2, dist + 16 * lane);\n      }\n";
    }
    s += "      __syncwarp();\n";
}

void emit_cut_masks(std::string& s, const Shape& sh) {
    for (int q = 0; q < sh.c; ++q) emitf(s, "      const int g%d = sg[cu%d] >> 4;\n", q, q);
}

// consts: empty for a function shared by a shape (values as parameters), else
// the one operation's values as constants
void emit_forward(std::string& s, const Shape& sh, int id, const std::string& consts) {
    const int ncell = 1 << (2 * sh.c), nitem = 4 * ncell;
    emitf(s,
          "// forward %d: %s\n"
          "__device__ __noinline__ void fwd%d(float* __restrict__ A, float* __restrict__ dist,\n"
          "    const unsigned char* __restrict__ sg, const float* __restrict__ spri, const u32* cL, const u32* cR,\n"
          "    float th, float an, float th2, float an2, int lane%s%s) {\n%s"
          "  const int v = lane & 3, grp = lane & ~3;\n  {\n",
          id, sh.key.c_str(), id, consts.empty() ? ", " : "", consts.empty() ? params(sh).c_str() : "",
          consts.c_str());
    emit_dists(s, sh);
    s += "      const float tv = spri[4 * (sg[pe] & 3) + v];\n";
    emit_cut_masks(s, sh);
    s += "      float mx = 0.0f;\n";
    emitf(s, "      for (int it0 = 0; it0 < %d; it0 += 32) {\n", nitem);
    s += "        const int cell = (it0 + lane) >> 2;\n        float term = 0.0f;\n";
    emitf(s, "        if (it0 + lane < %d && tv != 0.0f && %s) {\n", nitem, valid_expr(sh, "cell").c_str());
    emitf(s, "          const int ext = cell | (v << %d);\n", 2 * sh.c);
    emit_term(s, sh, "          ");
    s += "          term = tmp;\n        }\n";
    s += "        const float t0 = __shfl_sync(FULL, term, grp), t1 = __shfl_sync(FULL, term, grp + 1);\n"
         "        const float t2 = __shfl_sync(FULL, term, grp + 2), t3 = __shfl_sync(FULL, term, grp + 3);\n";
    emitf(s,
          "        if (v == 0 && it0 + lane < %d) {\n"
          "          const float total = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(0.0f, t0), t1), t2), t3);\n"
          "          A[mat + cell] = total;\n"
          "          mx = total > mx ? total : mx;\n"
          "        }\n      }\n",
          nitem);
    emitf(s,
          "      for (int dd = 16; dd >= 1; dd >>= 1) { const float o = __shfl_xor_sync(FULL, mx, dd); mx = o > mx ? o : mx; }\n"
          "      if (mx > 0.0f) {\n"
          "        const float f = scalbnf(1.0f, -ilogbf(mx));\n"
          "        for (int cell = lane; cell < %d; cell += 32) A[mat + cell] = A[mat + cell] * f;\n"
          "      }\n"
          "      __syncwarp();\n  }\n}\n",
          ncell);
}

void emit_backward(std::string& s, const Shape& sh, int id, const std::string& consts, int di) {
    emitf(s,
          "// backward %d: %s\n"
          "__device__ __noinline__ void bwd%d(const float* __restrict__ A, float* __restrict__ dist,\n"
          "    const unsigned char* __restrict__ sg, const float* __restrict__ spri, const u32* cL, const u32* cR,\n"
          "    float th, float an, float th2, float an2, int lane, signed char* assign, const double* sdraw,\n"
          "    int* status%s%s) {\n%s"
          "  const int v = lane & 3;\n  {\n",
          id, sh.key.c_str(), id, consts.empty() ? ", int di, " : "", consts.empty() ? params(sh).c_str() : "",
          consts.empty() ? "" : (consts + "  const int di = " + std::to_string(di) + ";\n  (void)mat;\n").c_str());
    emit_dists(s, sh);
    emit_cut_masks(s, sh);
    s += "      int cellidx = 0;\n      bool known = true;\n";
    for (int q = 0; q < sh.c; ++q)
        emitf(s, "      { const int a = assign[cu%d]; known = known && a >= 0; cellidx |= (a & 3) << %d; }\n", q,
              2 * q);
    s += "      float pv = 0.0f;\n";
    s += "      if (lane < 4 && known) {\n        const float tv = spri[4 * (sg[pe] & 3) + lane];\n";
    emitf(s, "        if (tv != 0.0f && %s) {\n", valid_expr(sh, "cellidx").c_str());
    emitf(s, "          const int ext = cellidx | (v << %d);\n", 2 * sh.c);
    emit_term(s, sh, "          ");
    s += "          pv = tmp;\n        }\n      }\n";
    emitf(s,
          "      const float p0 = __shfl_sync(FULL, pv, 0), p1 = __shfl_sync(FULL, pv, 1);\n"
          "      const float p2 = __shfl_sync(FULL, pv, 2), p3 = __shfl_sync(FULL, pv, 3);\n"
          "      if (lane == 0) {\n"
          "        if (!known) atomicCAS(status, 0, %d);\n"
          "        float pd[4] = {p0, p1, p2, p3};\n"
          "        const float tot = __fadd_rn(__fadd_rn(__fadd_rn(p0, p1), p2), p3);\n"
          "        if (tot != 0.0f)\n"
          "          for (int q = 0; q < 4; ++q) pd[q] = __fdiv_rn(pd[q], tot);\n"
          "        const double r = sdraw[di];\n"
          "        float acc = 0.0f;\n"
          "        int lastv = 0, pick = -1;\n"
          "        for (int q = 0; q < 4; ++q) {\n"
          "          acc = __fadd_rn(acc, pd[q]);\n"
          "          if (r < (double)acc) { pick = q; break; }\n"
          "          if (pd[q] != 0.0f) lastv = q;\n"
          "        }\n"
          "        assign[pe] = (signed char)(pick >= 0 ? pick : lastv);\n"
          "      }\n"
          "      __syncwarp();\n  }\n}\n",
          (int)ST_ILLEGAL_DG);
}

std::string source(const JitLsIn& in, int wpb) {
    const Layout Ly = layout(in);
    std::string s;
    s.reserve(4096 + (size_t)in.K * 3000);
    s += kPhiloxSrc;
    emitf(s,
          "\ntypedef unsigned int u32;\ntypedef unsigned long long u64;\n"
          "#define WPB %d\n#define FULL 0xffffffffu\n"
          "__device__ __forceinline__ int matA(int s) { return (s == 1 || s == 2) ? 1 : 0; }\n"
          "__device__ __forceinline__ int patA(int s) { return (s == 1 || s == 3) ? 1 : 0; }\n",
          wpb);
    // transmission distributions of one child's two meioses (ls_dist_one)
    s += "__device__ __forceinline__ void dist_one(int b0, const u32* cL, const u32* cR, float th, float an, float th2,\n"
         "                                         float an2, float* d) {\n"
         "  for (int side = 0; side < 2; ++side) {\n"
         "    const int b = b0 + side;\n"
         "    float* s = d + side * 8;\n"
         "    s[0] = 1.0f; s[1] = 0.0f; s[2] = 0.0f; s[3] = 1.0f;\n"
         "    float tmp0 = 0.5f, tmp1 = 0.5f;\n"
         "    if (cL) { const bool cross = ((cL[b >> 5] >> (b & 31)) & 1u) != 0u;\n"
         "              tmp0 = __fmul_rn(tmp0, cross ? th2 : an2); tmp1 = __fmul_rn(tmp1, cross ? an2 : th2); }\n"
         "    if (cR) { const bool cross = ((cR[b >> 5] >> (b & 31)) & 1u) != 0u;\n"
         "              tmp0 = __fmul_rn(tmp0, cross ? th : an); tmp1 = __fmul_rn(tmp1, cross ? an : th); }\n"
         "    const float total = __fadd_rn(tmp0, tmp1);\n"
         "    const float uau = __fdiv_rn(tmp1, total);\n"
         "    s[4] = uau; s[5] = __fsub_rn(1.0f, uau);\n"
         "    const float uua = __fdiv_rn(tmp0, total);\n"
         "    s[6] = uua; s[7] = __fsub_rn(1.0f, uua);\n"
         "  }\n"
         "}\n";
    // parents of every meiosis bit, for the indicator phase
    const int nb = 2 * in.Nnf;
    s += "__constant__ short kPar[" + std::to_string(nb > 0 ? nb : 1) + "] = {";
    for (int b = 0; b < nb; ++b) {
        const int i = in.F + (b >> 1);
        s += std::to_string((b & 1) ? in.father[i] : in.mother[i]);
        s += b + 1 < nb ? "," : "";
        if (b % 32 == 31) s += "\n";
    }
    if (nb == 0) s += "0";
    s += "};\n";
    // small functions keep NVRTC's optimiser (superlinear in a function's
    // size) fast: up to 150 operations, one per operation and pass with the
    // operation's values as constants (the fastest code); above, one per
    // operation shape and pass, the values passed in (a few dozen functions:
    // seconds to compile, a smaller instruction footprint, somewhat more
    // address arithmetic)
    const bool per_op = in.K <= 150;
    std::vector<int> shape_id(in.K);
    std::vector<std::string> keys;
    for (int k = 0; k < in.K; ++k) {
        const Shape sh = shape_of(in, in.ops[k]);
        if (per_op) {
            const std::string cp = const_prologue(in, in.ops[k], sh);
            emit_forward(s, sh, k, cp);
            emit_backward(s, sh, k, cp, in.K - 1 - k);
            shape_id[k] = k;
            continue;
        }
        int id = -1;
        for (size_t i = 0; i < keys.size(); ++i)
            if (keys[i] == sh.key) id = (int)i;
        if (id < 0) {
            id = (int)keys.size();
            keys.push_back(sh.key);
            emit_forward(s, sh, id, "");
            emit_backward(s, sh, id, "", 0);
        }
        shape_id[k] = id;
    }
    emitf(s,
          "extern \"C\" __global__ void __launch_bounds__(WPB * 32) sl_ls_jit(u32* dg, int first, int nchain,\n"
          "    const int* loci, int nloci, const double* u, long long ucs, long long uls, u64 seed, u64 iter,\n"
          "    const u64* key, const unsigned char* sel, int want, int* status, const unsigned char* geno,\n"
          "    const float* prior_f, const float* c_theta_f) {\n"
          "  extern __shared__ __align__(16) unsigned char smem[];\n"
          "  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;\n"
          "  unsigned char* wsm = smem + (size_t)warp * %zu;\n"
          "  float* A = (float*)wsm;\n"
          "  float* dist = (float*)(wsm + %zu);\n"
          "  signed char* assign = (signed char*)(wsm + %zu);\n"
          "  double* sdraw = (double*)(wsm + %zu);\n"
          "  unsigned char* sg = wsm + %zu;\n"
          "  u32* sL = (u32*)(wsm + %zu);\n"
          "  u32* sR = sL + %d;\n"
          "  float* spri = (float*)(wsm + %zu);\n"
          "  const long long ntask = (long long)nchain * nloci;\n"
          "  for (long long t = (long long)blockIdx.x * WPB + warp; t < ntask; t += (long long)gridDim.x * WPB) {\n"
          "    const int cr = (int)(t / nloci);\n"
          "    if (sel && sel[cr] != want) continue;\n"
          "    const int l = loci[t %% nloci];\n"
          "    const int chain = first + cr;\n"
          "    const bool hasL = l > 0, hasR = l < %d;\n"
          "    u32* colC = dg + ((long long)chain * %d + l) * %d;\n",
          Ly.total, Ly.dist, Ly.assign, Ly.draws, Ly.gcol, Ly.cols, in.W, Ly.pri, in.M - 1, in.M, in.W);
    emitf(s,
          "    {\n"
          "      const unsigned char* gsrc = geno + (long long)l * %d;\n"
          "      for (int i = lane; i < %d; i += 32) sg[i] = gsrc[i];\n"
          "      for (int w = lane; w < %d; w += 32) { if (hasL) sL[w] = colC[w - %d]; if (hasR) sR[w] = colC[w + %d]; }\n"
          "      if (lane < 16) spri[lane] = prior_f[(long long)l * 16 + lane];\n"
          "      __syncwarp();\n"
          "    }\n"
          "    const u32* cL = hasL ? sL : (const u32*)0;\n"
          "    const u32* cR = hasR ? sR : (const u32*)0;\n"
          "    float th = 1.0f, an = 1.0f, th2 = 1.0f, an2 = 1.0f;\n"
          "    { const float* tf = c_theta_f + (long long)chain * %d;\n"
          "      if (hasL) { th2 = tf[l - 1]; an2 = 1.0f - th2; }\n"
          "      if (hasR) { th = tf[l]; an = 1.0f - th; } }\n",
          in.N, in.N, in.W, in.W, in.W, in.M - 1);
    for (int k = 0; k < in.K; ++k)
        emitf(s, "    fwd%d(A, dist, sg, spri, cL, cR, th, an, th2, an2, lane%s%s);\n", shape_id[k],
              per_op ? "" : ", ", per_op ? "" : call_args(in, in.ops[k]).c_str());
    emitf(s,
          "    if (A[%d] == 0.0f) {\n"
          "      if (lane == 0) atomicCAS(status, 0, %d);\n"
          "      __syncwarp();\n"
          "      continue;\n"
          "    }\n"
          "    for (int i = lane; i < %d; i += 32) assign[i] = -1;\n"
          "    for (int j = lane; j < %d; j += 32) {\n"
          "      if (u) sdraw[j] = u[cr * ucs + l * uls + j];\n"
          "      else { const u64 sd = key ? key[0] : seed, it = key ? key[1] : iter;\n"
          "             sdraw[j] = sl_philox_u01(sd, ((u64)chain << 40) ^ (it << 4) ^ 1ull, ((u64)l << 24) ^ (u64)j); }\n"
          "    }\n"
          "    __syncwarp();\n",
          in.ops[in.K - 1].mat_off, (int)ST_ZERO_LIK, in.N, in.K);
    for (int k = in.K - 1; k >= 0; --k) {
        if (per_op)
            emitf(s, "    bwd%d(A, dist, sg, spri, cL, cR, th, an, th2, an2, lane, assign, sdraw, status);\n", k);
        else
            emitf(s, "    bwd%d(A, dist, sg, spri, cL, cR, th, an, th2, an2, lane, assign, sdraw, status, %d, %s);\n",
                  shape_id[k], in.K - 1 - k, call_args(in, in.ops[k]).c_str());
    }
    // meiosis indicators (locus_sampler2.cc:32-125)
    emitf(s,
          "    {\n"
          "      long long cursor = %d;\n"
          "      for (int w = 0; w < %d; ++w) {\n"
          "        const int b = 32 * w + lane;\n"
          "        int mi = 0, need = 0;\n"
          "        float p0 = 1.0f, p1 = 1.0f;\n"
          "        if (b < %d) {\n"
          "          const int i = %d + (b >> 1), par = b & 1;\n"
          "          const int tr = assign[i];\n"
          "          const int ptr = assign[kPar[b]];\n"
          "          const int allele = par == 0 ? ((tr == 0 || tr == 3) ? 0 : 1) : ((tr == 0 || tr == 2) ? 0 : 1);\n"
          "          if (ptr == 3 || ptr == 2) {\n"
          "            mi = allele == 0 ? (ptr == 3 ? 0 : 1) : (ptr == 3 ? 1 : 0);\n"
          "          } else {\n"
          "            need = 1;\n"
          "            if (hasL) { const int d = (sL[b >> 5] >> (b & 31)) & 1;\n"
          "                        p0 = __fmul_rn(p0, d == 0 ? an2 : th2); p1 = __fmul_rn(p1, d == 1 ? an2 : th2); }\n"
          "            if (hasR) { const int d = (sR[b >> 5] >> (b & 31)) & 1;\n"
          "                        p0 = __fmul_rn(p0, d == 0 ? an : th); p1 = __fmul_rn(p1, d == 1 ? an : th); }\n"
          "          }\n"
          "        }\n"
          "        const unsigned nmask = __ballot_sync(FULL, need);\n"
          "        if (need) {\n"
          "          const long long k = cursor + __popc(nmask & ((1u << lane) - 1u));\n"
          "          double r;\n"
          "          if (u) r = u[cr * ucs + l * uls + k];\n"
          "          else { const u64 sd = key ? key[0] : seed, it = key ? key[1] : iter;\n"
          "                 r = sl_philox_u01(sd, ((u64)chain << 40) ^ (it << 4) ^ 1ull, ((u64)l << 24) ^ (u64)k); }\n"
          "          mi = (r < (double)__fdiv_rn(p0, __fadd_rn(p0, p1))) ? 0 : 1;\n"
          "        }\n"
          "        cursor += __popc(nmask);\n"
          "        const unsigned word = __ballot_sync(FULL, mi != 0);\n"
          "        if (lane == 0) colC[w] = word;\n"
          "      }\n"
          "      __syncwarp();\n"
          "    }\n"
          "  }\n"
          "}\n",
          in.K, in.W, nb, in.F);
    return s;
}

}  // namespace

size_t jit_ls_warp_bytes(const JitLsIn& in) { return layout(in).total; }

std::string jit_ls_source(const JitLsIn& in, int wpb) { return source(in, wpb); }

int jit_ls_load(const JitBinary& bin, int wpb, size_t warp_bytes, JitLs* out, std::string* log) {
    *out = JitLs{};
    if (bin.rc) {
        *log = bin.log;
        return -1;
    }
    if (jit_load_kernel(bin.cubin, "sl_ls_jit", &out->lib, &out->kern, log)) return -1;
    out->wpb = wpb;
    out->smem = (size_t)wpb * warp_bytes;
    if (cudaFuncSetAttribute((const void*)out->kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)out->smem) !=
        cudaSuccess) {
        jit_ls_release(out);
        *log = "the specialised L-sampler's shared memory does not fit";
        return -1;
    }
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, (const void*)out->kern) == cudaSuccess) {
        out->regs = fa.numRegs;
        out->local_bytes = (int)fa.localSizeBytes;
    }
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, (const void*)out->kern, wpb * 32, out->smem) !=
            cudaSuccess ||
        blocks < 1) {
        jit_ls_release(out);
        *log = "the specialised L-sampler cannot be resident";
        return -1;
    }
    out->blocks_per_sm = blocks;
    return 0;
}

int jit_ls_compile(const JitLsIn& in, int wpb, JitLs* out, std::string* log) {
    const auto t0 = std::chrono::steady_clock::now();
    const std::shared_ptr<const JitBinary> bin = jit_binary(source(in, wpb), "sl_ls_jit.cu");
    if (jit_ls_load(*bin, wpb, layout(in).total, out, log)) return -1;
    out->compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

void jit_ls_release(JitLs* j) {
    if (j && j->lib) cudaLibraryUnload((cudaLibrary_t)j->lib);
    if (j) *j = JitLs{};
}

cudaError_t jit_ls_launch(const JitLs& j, uint32_t* dg, int first, int nchain, const int32_t* loci, int nloci,
                          const double* u, int64_t ucs, int64_t uls, uint64_t seed, uint64_t iter, const uint64_t* key,
                          const uint8_t* sel, int want, int* status, const uint8_t* geno, const float* prior_f,
                          const float* c_theta_f, int sms, cudaStream_t s) {
    const int64_t ntask = (int64_t)nchain * nloci;
    int64_t grid = (ntask + j.wpb - 1) / j.wpb;
    const int64_t cap = (int64_t)sms * j.blocks_per_sm;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    long long ucs_ = ucs, uls_ = uls;
    unsigned long long seed_ = seed, iter_ = iter;
    void* args[] = {(void*)&dg,   (void*)&first, (void*)&nchain, (void*)&loci,  (void*)&nloci, (void*)&u,
                    (void*)&ucs_, (void*)&uls_,  (void*)&seed_,  (void*)&iter_, (void*)&key,   (void*)&sel,
                    (void*)&want, (void*)&status, (void*)&geno,  (void*)&prior_f, (void*)&c_theta_f};
    return cudaLaunchKernel((const void*)j.kern, dim3((unsigned)grid), dim3(j.wpb * 32), args, j.smem, s);
}

}  // namespace sl
