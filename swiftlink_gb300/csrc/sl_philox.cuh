// Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): a counter-based uniform in [0, 1) from a 64-bit
// key and a 128-bit counter, 53 random bits per draw.  Plain types only: the
// same text is compiled into the library and into the kernels specialised at
// run time, so every kernel draws the same stream.
#pragma once

__device__ __forceinline__ double sl_philox_u01(unsigned long long key, unsigned long long c_hi,
                                                unsigned long long c_lo) {
    unsigned int c0 = (unsigned int)c_lo, c1 = (unsigned int)(c_lo >> 32);
    unsigned int c2 = (unsigned int)c_hi, c3 = (unsigned int)(c_hi >> 32);
    unsigned int k0 = (unsigned int)key, k1 = (unsigned int)(key >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned int hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const unsigned int hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const unsigned int n0 = hi1 ^ c1 ^ k0;
        const unsigned int n2 = hi0 ^ c3 ^ k1;
        c1 = lo1;
        c3 = lo0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    const unsigned long long hi = c0 >> 5, lo = c1 >> 6;
    return (double)(hi * 67108864ull + lo) * (1.0 / 9007199254740992.0);
}
