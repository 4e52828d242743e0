// The batched trait peel specialised to one problem.
//
// The host compiler of the trait peel (compile_lod_program in sl_host.cc)
// yields a slot program: LI_REC / LI_SUM / LI_CELL / LI_SCALE over float
// slots.  lod_prog_kernel interprets it, paying for every factor a program
// word load, an address computation and a shared-memory access.  Here the same
// program is written out as straight-line CUDA C++ (every slot a value in
// static single assignment, every constant an immediate, every indicator bit a
// shift of a register), compiled with NVRTC for sm_103a when the context is
// created, and loaded with cudaLibraryLoadData.  The arithmetic is the
// interpreter's, operation for operation (products left to right, sums in
// term order, the same power-of-two rescaling); only FMA contraction may fuse
// a product into the following sum.
//
// Two storage forms are generated: values in registers (the compiler
// allocates and, past its register budget, spills) and values in a per-thread
// shared-memory arena with immediate offsets.  Both are timed at creation and
// the faster kept (jit_lod_pick).
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sl_internal.h"
#include "sl_jit.h"

namespace sl {

namespace {

void emitf(std::string& s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void emitf(std::string& s, const char* fmt, ...) {
    char buf[512];
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

std::string flit(float c) {
    char buf[64];
    snprintf(buf, sizeof(buf), "%af", (double)c);   // hexadecimal: the exact float value
    return buf;
}

// Straight-line source of one problem's trait peel.
std::string jit_source(const JitProgramIn& in, int threads, bool shared) {
    std::string s;
    s.reserve(in.n_words * 24 + 4096);
    const int64_t npos = (int64_t)(in.M - 1) * in.n;
    emitf(s, "#define S %d\n", threads);
    s += "typedef unsigned int u32;\n";
    emitf(s,
          "extern \"C\" __global__ void __launch_bounds__(S) sl_lod_jit(const u32* __restrict__ graphs, long long gw,\n"
          "    int G, double* __restrict__ vals, int* status, const float* __restrict__ partial,\n"
          "    const double* __restrict__ lt_tab, const double* __restrict__ la_tab) {\n");
    if (shared) s += "  extern __shared__ float sh[];\n  float* A = sh + threadIdx.x;\n";
    emitf(s, "  const long long npos = %lldLL;\n", (long long)npos);
    s += "  const long long ntask = (long long)G * npos;\n";
    s += "  for (long long t = (long long)blockIdx.x * S + threadIdx.x; t < ntask; t += (long long)gridDim.x * S) {\n";
    emitf(s, "    const int b = (int)(t / npos);\n    const int pidx = (int)(t %% npos);\n");
    emitf(s, "    const int l = pidx / %d, o = pidx %% %d;\n", in.n, in.n);
    emitf(s, "    const u32* cL = graphs + (long long)b * gw + (long long)l * %d;\n    const u32* cR = cL + %d;\n", in.W,
          in.W);
    for (int w = 0; w < in.W; ++w) emitf(s, "    const u32 wL%d = cL[%d], wR%d = cR[%d];\n", w, w, w, w);
    emitf(s, "    const float th = partial[l] * (float)(o + 1), th2 = partial[l] * (float)(%d - o);\n", in.n);
    s += "    const float an = 1.0f - th, an2 = 1.0f - th2;\n";
    s += "    int scale = 0;\n";
    // slot -> current value name
    std::vector<int> cur;
    int next = 0;
    auto ref = [&](int slot) {
        std::string r;
        if (shared) {
            char b[48];
            snprintf(b, sizeof(b), "A[%d]", slot * threads);
            r = b;
        } else {
            if (slot >= (int)cur.size() || cur[slot] < 0) return std::string("0.0f");
            r = "v" + std::to_string(cur[slot]);
        }
        return r;
    };
    auto def = [&](int slot) {
        if (shared) {
            char b[48];
            snprintf(b, sizeof(b), "    A[%d] = ", slot * threads);
            return std::string(b);
        }
        if (slot >= (int)cur.size()) cur.resize(slot + 1, -1);
        cur[slot] = next++;
        return "    const float v" + std::to_string(cur[slot]) + " = ";
    };
    const int32_t* pc = in.words;
    const int32_t* end = in.words + in.n_words;
    int rec = 0, sc = 0;
    std::string result = "0.0f";
    while (pc < end) {
        const int op = pc[0];
        if (op == LI_CELL) {
            const int dst = pc[1], nt = pc[2];
            pc += 3;
            std::string e;
            for (int q = 0; q < nt; ++q) {
                const int nf = pc[0];
                std::string term = flit(in.consts[pc[1]]);
                pc += 2;
                for (int f = 0; f < nf; ++f) term = "(" + term + " * " + ref(pc[f]) + ")";
                pc += nf;
                e += (q ? " + " : "") + term;
            }
            if (nt == 0) e = "0.0f";
            s += def(dst) + e + ";\n";
        } else if (op == LI_REC) {
            const int child = pc[1], dst = pc[2];
            pc += 3;
            const int bpos = 2 * (child - in.F), w = bpos >> 5, bit = bpos & 31;
            const int r = rec++;
            emitf(s,
                  "    const unsigned mL%d = (wL%d >> %d) & 1u, pL%d = (wL%d >> %d) & 1u, mR%d = (wR%d >> %d) & 1u, "
                  "pR%d = (wR%d >> %d) & 1u;\n",
                  r, w, bit, r, w, bit + 1, r, w, bit, r, w, bit + 1);
            for (int k = 0; k < 4; ++k) {
                const int i = k >> 1, j = k & 1;
                // trait_rec: (bit == i ? an : th) for the locus, (bit == i ? an2 : th2) for locus + 1
                char e[256];
                snprintf(e, sizeof(e),
                         "0.25f * ((((mL%d == %du) ? an : th) * ((mR%d == %du) ? an2 : th2)) * ((pL%d == %du) ? an : th)"
                         " * ((pR%d == %du) ? an2 : th2))",
                         r, i, r, i, r, j, r, j);
                s += def(dst + k) + e + ";\n";
            }
        } else if (op == LI_SUM) {
            const int dst = pc[1], ns = pc[2];
            std::string e;
            for (int q = 0; q < ns; ++q) e += (q ? " + " : "") + ref(pc[3 + q]);
            if (ns == 0) e = "0.0f";
            s += def(dst) + e + ";\n";
            pc += 3 + ns;
        } else if (op == LI_SCALE) {
            const int first = pc[1], cnt = pc[2], target = pc[3];
            pc += 4;
            const int k = sc++;
            std::string mx = "0.0f";
            for (int q = 0; q < cnt; ++q) mx = "fmaxf(" + mx + ", " + ref(first + q) + ")";
            emitf(s, "    const float mx%d = %s;\n", k, mx.c_str());
            emitf(s, "    const int e%d = mx%d > 0.0f ? ilogbf(mx%d) - %d : 0;\n    scale += e%d;\n", k, k, k,
                  target, k);
            // 2^-e as a float when it is a normal number (nearly always): a product
            // with it is exact, or rounded once where the result is subnormal, as
            // ldexpf rounds; ldexpf only where 2^-e itself is out of range
            emitf(s, "    const float sc%d = (e%d >= -127 && e%d <= 126) ? __int_as_float((127 - e%d) << 23) : 0.0f;\n",
                  k, k, k, k);
            std::vector<std::string> olds(cnt), news(cnt);
            for (int q = 0; q < cnt; ++q) olds[q] = ref(first + q);
            if (shared) {
                for (int q = 0; q < cnt; ++q) news[q] = olds[q];
            } else {
                std::string decl = "    float ";
                for (int q = 0; q < cnt; ++q) {
                    const int slot = first + q;
                    if (slot >= (int)cur.size()) cur.resize(slot + 1, -1);
                    cur[slot] = next++;
                    news[q] = "v" + std::to_string(cur[slot]);
                    decl += (q ? ", " : "") + news[q];
                }
                s += decl + ";\n";
            }
            emitf(s, "    if (sc%d != 0.0f) {\n", k);
            for (int q = 0; q < cnt; ++q) emitf(s, "      %s = %s * sc%d;\n", news[q].c_str(), olds[q].c_str(), k);
            s += "    } else {\n";
            for (int q = 0; q < cnt; ++q)
                emitf(s, "      %s = ldexpf(%s, -e%d);\n", news[q].c_str(), olds[q].c_str(), k);
            s += "    }\n";
        } else {   // LI_END
            const int rs = pc[1];
            result = rs >= 0 ? ref(rs) : std::string("0.0f");
            break;
        }
    }
    emitf(s, "    const float result = %s;\n", result.c_str());
    s += "    int cross = 0;\n";
    for (int w = 0; w < in.W; ++w) emitf(s, "    cross += __popc(wL%d ^ wR%d);\n", w, w);
    emitf(s, "    const double rec = cross * lt_tab[l] + (%d - cross) * la_tab[l];\n", 2 * in.Nnf);
    s += "    double v;\n";
    emitf(s,
          "    if (!(result > 0.0f)) { %s v = -1.7976931348623157e308; }\n"
          "    else v = (double)logf(result) + (double)scale * 0.69314718055994530942 - rec - (%.17g);\n",
          in.zero_ok ? "" : ("atomicCAS(status, 0, " + std::to_string((int)ST_LOD_NONPOS) + ");").c_str(),
          in.marker_trans);
    s += "    vals[t] = v;\n  }\n}\n";
    return s;
}

}  // namespace

namespace {

// NVRTC for sm_103a: source to cubin, no CUDA context needed.
int nvrtc_cubin(const std::string& src, const char* file, std::vector<char>* cubin, std::string* log) {
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), file, 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        *log = "nvrtcCreateProgram failed";
        return -1;
    }
    const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device"};
    nvrtcResult r = nvrtcCompileProgram(prog, 3, opts);
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    if (ls > 1) {
        std::string l(ls, '\0');
        nvrtcGetProgramLog(prog, &l[0]);
        *log += l;
    }
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        *log = std::string("nvrtc: ") + nvrtcGetErrorString(r) + "\n" + *log;
        return -1;
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin->resize(n);
    nvrtcGetCUBIN(prog, cubin->data());
    nvrtcDestroyProgram(&prog);
    return 0;
}

// Compiles running at once: each takes a core and up to a few hundred MB,
// and a program may ask for one per pedigree.
class CompileSlots {
  public:
    CompileSlots() {
        const unsigned hw = std::thread::hardware_concurrency();
        free_ = hw >= 4 ? (int)std::min(8u, hw / 2) : 2;
    }
    void take() {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return free_ > 0; });
        --free_;
    }
    void give() {
        { std::lock_guard<std::mutex> lk(mu_); ++free_; }
        cv_.notify_one();
    }

  private:
    std::mutex mu_;
    std::condition_variable cv_;
    int free_;
};

struct BinaryCache {
    std::mutex mu;
    std::condition_variable cv;
    std::list<std::shared_ptr<JitBinary>> lru;   // most recent first
    CompileSlots slots;
};

BinaryCache& binary_cache() {
    static BinaryCache* c = new BinaryCache();   // never destroyed: background compiles may outlive main
    return *c;
}

constexpr size_t kCachedBinaries = 32;

}  // namespace

std::shared_ptr<const JitBinary> jit_binary(const std::string& src, const char* file) {
    BinaryCache& c = binary_cache();
    std::shared_ptr<JitBinary> job;
    {
        std::unique_lock<std::mutex> lk(c.mu);
        for (auto it = c.lru.begin(); it != c.lru.end(); ++it)
            if ((*it)->source == src) {
                job = *it;
                c.lru.splice(c.lru.begin(), c.lru, it);
                break;
            }
        if (!job) {
            job = std::make_shared<JitBinary>();
            job->source = src;
            c.lru.push_front(job);
            while (c.lru.size() > kCachedBinaries) c.lru.pop_back();
        } else {
            // another caller compiles this source: wait for its result
            c.cv.wait(lk, [&] { return job->done; });
            return job;
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    c.slots.take();
    std::vector<char> cubin;
    std::string log;
    const int rc = nvrtc_cubin(src, file, &cubin, &log);
    c.slots.give();
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        job->cubin.swap(cubin);
        job->log = log;
        job->rc = rc;
        job->compile_ms = ms;
        job->done = true;
        if (rc) c.lru.remove(job);   // a failure is reported once, not cached
    }
    c.cv.notify_all();
    return job;
}

int jit_load_kernel(const std::vector<char>& cubin, const char* kernel, void** lib_out, void** kern_out,
                    std::string* log) {
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        *log = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e);
        return -1;
    }
    cudaKernel_t k = nullptr;
    e = cudaLibraryGetKernel(&k, lib, kernel);
    if (e != cudaSuccess) {
        cudaLibraryUnload(lib);
        *log = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e);
        return -1;
    }
    *lib_out = lib;
    *kern_out = (void*)k;
    return 0;
}

int jit_compile_kernel(const std::string& src, const char* file, const char* kernel, void** lib_out, void** kern_out,
                       std::string* log) {
    const std::shared_ptr<const JitBinary> bin = jit_binary(src, file);
    if (bin->rc) {
        *log = bin->log;
        return -1;
    }
    return jit_load_kernel(bin->cubin, kernel, lib_out, kern_out, log);
}

std::string jit_lod_source(const JitProgramIn& in, int threads, bool shared) {
    return jit_source(in, threads, shared);
}

int jit_lod_compile(const JitProgramIn& in, int threads, bool shared, JitLod* out, std::string* log) {
    *out = JitLod{};
    const auto t0 = std::chrono::steady_clock::now();
    const std::string src = jit_source(in, threads, shared);
    if (jit_compile_kernel(src, shared ? "sl_lod_jit_smem.cu" : "sl_lod_jit_reg.cu", "sl_lod_jit", &out->lib,
                           &out->kern, log))
        return -1;
    out->threads = threads;
    out->shared = shared;
    out->smem = shared ? (size_t)threads * in.slots * sizeof(float) : 0;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, (const void*)out->kern) == cudaSuccess) {
        out->regs = fa.numRegs;
        out->local_bytes = (int)fa.localSizeBytes;
    }
    if (out->smem > 0 &&
        cudaFuncSetAttribute((const void*)out->kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)out->smem) !=
            cudaSuccess) {
        jit_lod_release(out);
        *log = "shared-memory arena does not fit";
        return -1;
    }
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, (const void*)out->kern, threads, out->smem) !=
            cudaSuccess ||
        blocks < 1) {
        jit_lod_release(out);
        *log = "specialised LOD kernel cannot be resident";
        return -1;
    }
    out->blocks_per_sm = blocks;
    out->compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

void jit_lod_release(JitLod* j) {
    if (j && j->lib) cudaLibraryUnload((cudaLibrary_t)j->lib);
    if (j) *j = JitLod{};
}

cudaError_t jit_lod_launch(const JitLod& j, const uint32_t* graphs, int64_t graph_words, int G, double* vals,
                           int* status, const float* partial, const double* lt, const double* la, int64_t ntask,
                           int sms, cudaStream_t s) {
    int64_t grid = (ntask + j.threads - 1) / j.threads;
    const int64_t cap = (int64_t)sms * j.blocks_per_sm * 4;
    if (grid > cap) grid = cap;
    long long gw = graph_words;
    void* args[] = {(void*)&graphs, (void*)&gw, (void*)&G, (void*)&vals, (void*)&status, (void*)&partial,
                    (void*)&lt, (void*)&la};
    return cudaLaunchKernel((const void*)j.kern, dim3((unsigned)grid), dim3(j.threads), args, j.smem, s);
}

}  // namespace sl
