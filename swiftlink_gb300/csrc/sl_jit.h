// The batched trait peel specialised to one problem at context creation
// (straight-line CUDA C++ compiled with NVRTC); see sl_jit.cc.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace sl {

// One compiled slot program and the sizes its source needs.
struct JitProgramIn {
    const int32_t* words;
    size_t n_words;
    const float* consts;
    int F, M, n, W, Nnf, slots;
    double marker_trans;
    int zero_ok;             // a zero trait likelihood is a zero term, not an error
};

struct JitLod {
    void* lib = nullptr;     // cudaLibrary_t
    void* kern = nullptr;    // cudaKernel_t
    int threads = 0;
    bool shared = false;     // values in a shared-memory arena (else registers)
    size_t smem = 0;
    int regs = 0;
    int local_bytes = 0;     // spill space per thread
    int blocks_per_sm = 0;
    double compile_ms = 0.0;
};

// One NVRTC compile of a source for sm_103a.
struct JitBinary {
    std::string source;
    std::vector<char> cubin;
    std::string log;
    int rc = -1;             // 0: cubin holds the binary
    double compile_ms = 0.0;
    bool done = false;
};

// The cubin of `src`, compiled on the calling thread (no CUDA context is
// needed) or taken from a process-wide cache of recent sources; a caller
// asking for a source another thread is compiling waits for that compile.
// At most a few compiles run at once.  Thread-safe.
std::shared_ptr<const JitBinary> jit_binary(const std::string& src, const char* file);

// Load `kernel` from a cubin into the current device's context (a
// cudaLibrary_t and a cudaKernel_t); 0 on success, else -1 with the reason.
int jit_load_kernel(const std::vector<char>& cubin, const char* kernel, void** lib, void** kern, std::string* log);

// jit_binary, then jit_load_kernel.
int jit_compile_kernel(const std::string& src, const char* file, const char* kernel, void** lib, void** kern,
                       std::string* log);

std::string jit_lod_source(const JitProgramIn& in, int threads, bool shared);
int jit_lod_compile(const JitProgramIn& in, int threads, bool shared, JitLod* out, std::string* log);
void jit_lod_release(JitLod* j);
cudaError_t jit_lod_launch(const JitLod& j, const uint32_t* graphs, int64_t graph_words, int G, double* vals,
                           int* status, const float* partial, const double* lt, const double* la, int64_t ntask,
                           int sms, cudaStream_t s);

}  // namespace sl
