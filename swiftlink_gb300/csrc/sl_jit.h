// The batched trait peel specialised to one problem at context creation
// (straight-line CUDA C++ compiled with NVRTC); see sl_jit.cc.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

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

// NVRTC-compile `src` for sm_103a and load `kernel` from it (a cudaLibrary_t
// and a cudaKernel_t); 0 on success, else -1 with the reason in *log.
int jit_compile_kernel(const std::string& src, const char* file, const char* kernel, void** lib, void** kern,
                       std::string* log);

std::string jit_lod_source(const JitProgramIn& in, int threads, bool shared);
int jit_lod_compile(const JitProgramIn& in, int threads, bool shared, JitLod* out, std::string* log);
void jit_lod_release(JitLod* j);
cudaError_t jit_lod_launch(const JitLod& j, const uint32_t* graphs, int64_t graph_words, int G, double* vals,
                           int* status, const float* partial, const double* lt, const double* la, int64_t ntask,
                           int sms, cudaStream_t s);

}  // namespace sl
