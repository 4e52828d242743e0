// TEST INFRASTRUCTURE ONLY (part of the oracle, never shipped or measured).
//
// Replacement for the reference's RNG translation unit (random.cc:1-99), so
// the reference's own CPU sources can be compiled here without GSL and fed
// caller-chosen uniform draws.  It provides the six functions declared in the
// reference's random.h:12-17.
//
//  * get_random(): when an injection buffer is armed, returns its values in
//    order (the reference consumes draws strictly sequentially within one
//    sampler step); otherwise draws from a seeded std::mt19937.
//  * get_random_int(limit): always from the seeded generator (peel-sequence
//    search, random descent graph, sequential imputation start locus).
//
// The GSL stream itself is not reproduced: parity is defined on injected
// uniforms, not on GSL's sequence.

#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>

using namespace std;

namespace {
std::mt19937 g_gen(12345u);
const double* g_buf = nullptr;
int g_len = 0;
int g_pos = 0;
int g_overrun = 0;
}  // namespace

extern "C" void stub_seed(unsigned int seed) { g_gen.seed(seed); }

extern "C" void stub_arm(const double* buf, int len) {
    g_buf = buf;
    g_len = len;
    g_pos = 0;
    g_overrun = 0;
}

extern "C" int stub_disarm() {
    int used = g_pos;
    g_buf = nullptr;
    g_len = 0;
    g_pos = 0;
    return g_overrun ? -1 : used;
}

void init_random() {}
void destroy_random() {}
void seed_random_explicit(string) {}
void seed_random_implicit() {}

double get_random() {
    if (g_buf) {
        if (g_pos < g_len) return g_buf[g_pos++];
        g_overrun = 1;
        return 0.5;
    }
    // 53-bit uniform in [0, 1)
    unsigned long long a = g_gen() >> 5, b = g_gen() >> 6;
    return (double)(a * 67108864ull + b) * (1.0 / 9007199254740992.0);
}

int get_random_int(int limit) {
    std::uniform_int_distribution<int> d(0, limit - 1);
    return d(g_gen);
}
