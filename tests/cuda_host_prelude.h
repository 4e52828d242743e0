// Definitions under which a generated CUDA kernel of this library compiles as
// plain host C++ (test harness only): qualifiers expand to nothing, the
// builtins it calls are written out, and the thread and block indices are
// variables that the caller's loop sets before each call.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <math.h>
#define __device__
#define __noinline__
#define __forceinline__ inline
#define __restrict__
#define __global__
#define __launch_bounds__(...)
struct float4 {
    float x, y, z, w;
};
struct host_dim {
    unsigned x;
};
static host_dim blockIdx, threadIdx, gridDim;
inline float __int_as_float(int i) {
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
inline double __longlong_as_double(long long i) {
    double d;
    std::memcpy(&d, &i, 8);
    return d;
}
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int atomicCAS(int* p, int c, int v) {
    const int o = *p;
    if (o == c) *p = v;
    return o;
}
