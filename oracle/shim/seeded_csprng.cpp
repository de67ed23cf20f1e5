// seeded_csprng.cpp -- replacement translation unit for the reference's ChaCha20Rng
// (declared in yatfhe/include/yatfhe/csprng.h:11-28, defined in yatfhe/src/csprng.cpp).
// TEST INFRASTRUCTURE ONLY.  The reference seeds every thread_local instance from
// getrandom() (yatfhe/src/csprng.cpp:63-72), so nothing it generates is reproducible;
// the oracle build compiles this file in place of csprng.cpp so that keys, ciphertexts
// and fixtures follow from a seed.
//
// Seeding rule (the plain-C restatement in oracle/pbs_oracle.c follows the same rule):
//   key words 0,1 = low, high 32 bits of the 64-bit seed; key words 2..7 = 0;
//   64-bit block counter starts at 0; nonce = (stream id, 0), where the stream id is
//   the number of ChaCha20Rng instances constructed before this one in the process.
// The seed comes from yatfhe_oracle_set_seed() if it was called before the first
// instance is built, else from the YATFHE_SEED environment variable, else 0.
// The block function is ChaCha20 as published in RFC 8439 section 2.3 (20 rounds).
#include "yatfhe/csprng.h"

#include <atomic>
#include <cstdlib>

namespace {
std::atomic<uint32_t> g_stream_counter{0};
std::atomic<bool> g_seed_set{false};
uint64_t g_seed = 0;

uint64_t current_seed() {
    if (!g_seed_set.load()) {
        const char* env = std::getenv("YATFHE_SEED");
        g_seed = env ? std::strtoull(env, nullptr, 0) : 0;
        g_seed_set.store(true);
    }
    return g_seed;
}

inline uint32_t rotl32(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }

inline void qround(uint32_t* s, int a, int b, int c, int d) {
    s[a] += s[b]; s[d] ^= s[a]; s[d] = rotl32(s[d], 16);
    s[c] += s[d]; s[b] ^= s[c]; s[b] = rotl32(s[b], 12);
    s[a] += s[b]; s[d] ^= s[a]; s[d] = rotl32(s[d], 8);
    s[c] += s[d]; s[b] ^= s[c]; s[b] = rotl32(s[b], 7);
}
}  // namespace

extern "C" void yatfhe_oracle_set_seed(uint64_t seed) {
    g_seed = seed;
    g_seed_set.store(true);
    g_stream_counter.store(0);
}

ChaCha20Rng::ChaCha20Rng() {
    const uint64_t seed = current_seed();
    state_[0] = 0x61707865u;
    state_[1] = 0x3320646eu;
    state_[2] = 0x79622d32u;
    state_[3] = 0x6b206574u;
    state_[4] = static_cast<uint32_t>(seed);
    state_[5] = static_cast<uint32_t>(seed >> 32);
    for (int i = 6; i < 12; i++) state_[i] = 0;
    state_[12] = 0;
    state_[13] = 0;
    state_[14] = g_stream_counter.fetch_add(1);
    state_[15] = 0;
}

void ChaCha20Rng::refill() {
    uint32_t x[16];
    for (int i = 0; i < 16; i++) x[i] = state_[i];
    for (int r = 0; r < 10; r++) {
        qround(x, 0, 4, 8, 12);
        qround(x, 1, 5, 9, 13);
        qround(x, 2, 6, 10, 14);
        qround(x, 3, 7, 11, 15);
        qround(x, 0, 5, 10, 15);
        qround(x, 1, 6, 11, 12);
        qround(x, 2, 7, 8, 13);
        qround(x, 3, 4, 9, 14);
    }
    for (int i = 0; i < 16; i++) block_[i] = x[i] + state_[i];
    if (++state_[12] == 0) ++state_[13];
    blockPos_ = 0;
}

ChaCha20Rng::result_type ChaCha20Rng::operator()() {
    if (blockPos_ == 16) refill();
    return block_[blockPos_++];
}
