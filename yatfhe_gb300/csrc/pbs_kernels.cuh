// pbs_kernels.cuh -- the bootstrap kernels (declarations shared by the .cu and the host).
#pragma once
#include <cstddef>
#include <cstdint>

#include "rns.cuh"

namespace yg {

// Everything one launch of the blind-rotation kernel needs.
struct BrArgs {
    const int32_t* lwe_in;   // [count][n+1], or null when scaled_in is given
    const int32_t* scaled_in;// [count][n] mask already switched to mod 2N (ScaledTlwe::a), or null
    const int64_t* lut;      // [N] torus test polynomial, or null when acc_in is given
    const int64_t* acc_in;   // [count][(k+1) N] starting accumulator, or null
    const uint4* key;        // device BSK, slot layout (see key_slot_words)
    int32_t* big_out;        // [count][k N + 1] extracted LWE, or null
    int64_t* acc_out;        // [count][(k+1) N] accumulator, or null
    int count;
    int n;                   // LWE dimension
    int steps;               // CMux steps to run (n for a full blind rotation)
    int L;                   // gadget levels
    int radix_bits;
    Chan ch[kChannels];
    Crt crt;
};

struct KsArgs {
    const int32_t* big_in;   // [count][kN + 1]
    const int32_t* ksk;      // [kN][t][n+1]
    int32_t* out;            // [count][n+1]
    int count;
    int kN;
    int n;
    int t;
    int ks_radix_bits;
};

struct KeyConvArgs {
    const uint32_t* residues;  // [polys][3][N] coefficient residues
    uint32_t* key;             // device BSK in slot layout
    int polys;
    Chan ch[kChannels];
    uint32_t scale[kChannels];    // N^-1 2^32 mod p_c
    uint32_t scale_s[kChannels];  // Shoup companions
};

// u32 words of one (step, level, row, channel) block of the device key: 2 output polys.
__host__ __device__ inline size_t key_block_words(int N) { return 2 * (size_t)N; }
__host__ __device__ inline size_t key_words(int n, int L, int N) {
    return (size_t)n * L * 2 * kChannels * key_block_words(N);
}

size_t br_smem_bytes(int logN, int torus_bits, int n, int L);
int launch_keyconv(int logN, const KeyConvArgs& a, void* stream);
int launch_blind_rotate(int logN, int torus_bits, const BrArgs& a, void* stream);
int launch_keyswitch(const KsArgs& a, void* stream);

}  // namespace yg
