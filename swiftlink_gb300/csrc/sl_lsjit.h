// The FP32 L-sampler specialised to one pedigree (straight-line operations,
// NVRTC); see sl_lsjit.cc.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "sl_internal.h"
#include "sl_jit.h"

namespace sl {

struct JitLsIn {
    const OpDev* ops;        // host copies of the operation descriptors
    const int32_t* opdata;   // and their lists
    int K, N, F, M, W, Nnf, arena, max_child;
    const int32_t* mother;   // [N], -1 for founders
    const int32_t* father;
};

struct JitLs {
    void* lib = nullptr;     // cudaLibrary_t
    void* kern = nullptr;    // cudaKernel_t
    int wpb = 0;             // warps per block
    size_t smem = 0;
    int regs = 0;
    int local_bytes = 0;
    int blocks_per_sm = 0;
    double compile_ms = 0.0;
};

size_t jit_ls_warp_bytes(const JitLsIn& in);
std::string jit_ls_source(const JitLsIn& in, int wpb);
// Source, compile (through the process-wide cache) and load.
int jit_ls_compile(const JitLsIn& in, int wpb, JitLs* out, std::string* log);
// Load a compiled source (jit_binary of jit_ls_source) into the current
// device's context; warp_bytes = jit_ls_warp_bytes of the same input.
int jit_ls_load(const JitBinary& bin, int wpb, size_t warp_bytes, JitLs* out, std::string* log);
void jit_ls_release(JitLs* j);
cudaError_t jit_ls_launch(const JitLs& j, uint32_t* dg, int first, int nchain, const int32_t* loci, int nloci,
                          const double* u, int64_t ucs, int64_t uls, uint64_t seed, uint64_t iter, const uint64_t* key,
                          const uint8_t* sel, int want, int* status, const uint8_t* geno, const float* prior_f,
                          const float* c_theta_f, int sms, cudaStream_t s);

}  // namespace sl
