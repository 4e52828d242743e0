// The trait-peel adjoint specialised to one pedigree's peel (NVRTC); see
// sl_adjjit.cc.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "sl_internal.h"

namespace sl {

// The peel the adjoint is generated from: the context's operations with
// their opdata (the unpruned peel, every cell of every rfunction).
struct AdjJitIn {
    const OpDev* ops;
    int K;
    const int32_t* od;
    int F, M, n, W;
    int min_blocks;          // resident blocks of kAdjJitThreads per SM the kernel is compiled for
};

constexpr int kAdjJitThreads = 128;   // threads per block of the generated kernel
// the variants compiled and timed: 4 blocks per SM (128 registers a thread)
// or 8 (64 registers, more spills, twice the tasks in flight)
constexpr int kAdjJitVariants = 2;
constexpr int kAdjJitMinBlocks[kAdjJitVariants] = {4, 8};

struct AdjJit {
    void* lib = nullptr;     // cudaLibrary_t
    void* kern = nullptr;    // cudaKernel_t
    int half = 0;            // floats of one task's matrices (its adjoints take as many)
    int shapes = 0;          // distinct operation shapes: one forward and one reverse function each
    int regs = 0;
    int local_bytes = 0;
    int blocks_per_sm = 0;
    int min_blocks = 0;
    double compile_ms = 0.0;
};

// Floats of one block's arena: every task's matrices, adjoints and exponents
// for kAdjJitThreads resident tasks.
inline int64_t adj_jit_block_floats(int half, int K) { return (int64_t)(2 * half + K) * kAdjJitThreads; }

std::string adj_jit_source(const AdjJitIn& in, int* shapes, int* half);
int adj_jit_compile(const AdjJitIn& in, AdjJit* out, std::string* log);
void adj_jit_release(AdjJit* j);
// blocks: the grid, each block with its own arena slice (arena holds
// blocks * adj_jit_block_floats floats).
cudaError_t adj_jit_launch(const AdjJit& j, const uint32_t* graphs, int64_t graph_words, int64_t task0,
                           int64_t ntask, double* grad, int* status, const float* partial, float* arena,
                           int64_t blocks, const float* dprob, const float4* dgrad, int zero_ok, cudaStream_t s);

}  // namespace sl
