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
    const uint4* key;        // device BSK, slot layout (see key_block_words)
    // Multi-key batches: ciphertext c uses key_table[key_of[c]] and lut_table[lut_of[c]]
    // when the index arrays are given (then `key` / `lut` are ignored).
    const uint4* const* key_table;
    const int32_t* key_of;
    const int64_t* const* lut_table;
    const int32_t* lut_of;
    int32_t* big_out;        // [count][k N + 1] extracted LWE, or null
    int64_t* acc_out;        // [count][(k+1) N] accumulator, or null
    int count;
    int grid;                // CTAs to launch (0: enough for the batch; fewer: persistent CTAs)
    int per_cta;             // ciphertexts per CTA, sharing its L1 (1, 2 or 4; 0 means 1)
    int layout;              // kLayoutChannel, kLayoutChannelRow, kLayoutRowCluster or kLayoutChannelCluster
    int n;                   // LWE dimension
    int steps;               // CMux steps to run (n for a full blind rotation)
    int L;                   // gadget levels
    int radix_bits;
    Chan ch[kChannels];
    Crt crt;
    const uint2* tw16;       // [3][N] psi^-e mod p_c with Shoup companions (ntt16_inverse), or null
};

// A run of at most kKsTileCts consecutive ciphertexts of a batch that share one KSK.
struct KsTile {
    int ct_begin;
    int count;
    const int32_t* ksk;
};
constexpr int kKsTileCts = 8;

struct KsArgs {
    const int32_t* big_in;   // [count][kN + 1]
    const int32_t* ksk;      // [kN][t][n+1]
    int32_t* out;            // [count][n+1]
    int count;
    int kN;
    int n;
    int t;
    int ks_radix_bits;
    const KsTile* tiles;     // multi-key batches: one tile per block (then `ksk` is ignored)
    int num_tiles;
};

struct KeyConvArgs {
    const uint32_t* residues;  // [polys][3][N] coefficient residues
    uint32_t* key;             // device BSK in slot layout
    int polys;
    Chan ch[kChannels];
    uint32_t scale[kChannels];    // N^-1 2^32 mod p_c
    uint32_t scale_s[kChannels];  // Shoup companions
};

// The key loader's first step, on the GPU: the inverse negacyclic transform mod q of each
// NTT-domain key polynomial (the convention of the host's QInverse: Gentleman-Sande with
// psi^-brv(k) twiddles and Shoup companions, bit-reversed slots in, natural coefficients
// out, times N^-1), then each coefficient's centred representative reduced mod the three
// RNS primes.  One CTA per polynomial.
struct KeyInttArgs {
    const uint64_t* words;  // [polys][N] NTT-domain words mod q
    uint32_t* residues;     // [polys][3][N] centred coefficient residues mod p_c
    const uint64_t* w;      // [N] psi^-brv(k) mod q
    const uint64_t* wp;     // [N] floor(w 2^64 / q)
    uint64_t q, ninv, ninvp;
    uint32_t p[kChannels];
    int N, polys;
    int* bad;               // set to 1 when a word is not reduced mod q
};

// The GINX rows the WWL+24 blind rotation derives from its half key (cPrime rows and the s2
// key, both NTT-domain words mod q), written as NTT-domain BSK words [n][L][row][poly][N]
// for the key conversion above.  One CTA per (key index, level); k = 1.
constexpr int kWwlMaxLevels = 8;  // digit levels of the s2 key handled by the kernel
struct WwlExpandArgs {
    const uint64_t* cprime;  // [n][L][2][N]
    const uint64_t* s2;      // [Ls][2][N]
    const uint64_t* s2p;     // [Ls][2][N] floor(s2 2^64 / q)
    uint64_t* out;           // [n][L][2][2][N]
    const uint64_t* wi;      // [N] psi^-brv(k) mod q, and Shoup companions
    const uint64_t* wip;
    const uint64_t* wf;      // [N] psi^brv(k) mod q, and Shoup companions
    const uint64_t* wfp;
    uint64_t q, ninv, ninvp;
    int n, N, L, Ls, radix_bits, torus_bits;
    int* bad;                // set to 1 when a word is not reduced mod q
};

// Key generation from caller-drawn samples: the arithmetic of encryptTrgswMPNtt
// (yatfhe/src/trgsw.cpp:36-51, per key index of genBootstrappingKeyMP) and of
// genTlweKeySwitchingKey (yatfhe/src/keyswitching.cpp:19-29).  One CTA per BSK row sample
// (key index, level, row; row k is cPrime), N/2 threads; one warp per KSK sample.
struct KeygenBskArgs {
    const int32_t* lwe_s;     // [n] 0/1
    const int32_t* noise;     // [n][L][k+1][N] TUniform noise of each sample's b (torus)
    const uint64_t* mask;     // [n][L][k+1][k][N] uniform NTT-domain masks (< q)
    const uint64_t* s_ntt;    // [k][N] NTT of the RLWE secret mod q, and Shoup companions
    const uint64_t* s_ntt_p;
    const uint64_t* wf;       // [N] psi^brv(k) mod q, and Shoup companions
    const uint64_t* wfp;
    uint64_t* words;          // [n][L][k+1][k+1][N] NTT-domain BSK words
    uint64_t q;
    int n, N, k, L, radix_bits, torus_bits;
    int* bad;                 // set to 1 when a mask word is not reduced mod q
};
// Randomness drawn on the GPU (sampling.cu): `count` values of one kind from the ChaCha20
// stream of (seed, domain, stream).
constexpr int kDrawBit = 0;       // 0/1, one per word
constexpr int kDrawU32 = 1;       // uniform 32-bit words
constexpr int kDrawTUniform = 2;  // TUniform(b), 64 bits each
constexpr int kDrawModQ = 3;      // uniform mod q, 128 bits each
struct DrawArgs {
    int32_t* out_i32;   // kDrawBit, kDrawU32, kDrawTUniform
    uint64_t* out_u64;  // kDrawModQ
    uint64_t count;
    uint64_t seed;
    uint64_t q;
    uint32_t domain, stream;
    int kind, b;
    int per_block;      // values per 64-byte block: 16, 16, 8, 4
};
// symEncTlwe on `count` ciphertexts: masks and noise drawn (seed, domain, call) or given.
struct EncryptArgs {
    const int32_t* s;      // [n] binary LWE secret
    const int64_t* mu;     // [count] messages (torus, mod 2^32)
    const int32_t* mask;   // [count][n] or null (drawn)
    const int32_t* noise;  // [count] or null (drawn, TUniform(noise_b))
    int32_t* out;          // [count][n + 1]
    uint64_t seed;
    uint32_t domain, call;
    int count, n, noise_b;
};
// symEncTrlweMultiSampleSimple on `count` torus polynomials: NTT-domain samples [a_r | b].
struct EncryptRlweArgs {
    const int32_t* s;       // [k][N] binary RLWE secret
    const int64_t* mu;      // [count][N] torus plaintext coefficients
    const int32_t* noise;   // [count][N] TUniform noise
    const uint64_t* mask;   // [count][k][N] uniform NTT-domain masks (< q)
    uint64_t* out;          // [count][k+1][N]
    const uint64_t* wf;     // [N] psi^brv(k) mod q, and Shoup companions
    const uint64_t* wfp;
    uint64_t q, qinv, r2;   // q^-1 mod 2^64, 2^128 mod q
    int count, N, k, torus_bits, ctas;
    int* bad;               // set to 1 when a mask word is not reduced mod q (may be null)
};
int launch_encrypt_rlwe_ntt(const EncryptRlweArgs& a, void* stream);
// Approximate-CRT blind rotation (crt_kernels.cu): four residue primes, two high digits.
constexpr int kCrtD = 4, kCrtDh = 2;
struct CrtKeyConvArgs {
    const int8_t* bsk8;      // [n][d][dh][2 rows][2 polys][N] residues (int8, centred mod q_d)
    uint32_t* key;           // [n][d][dh][2 rows] blocks of key_block_words(N)
    Chan ch;                 // prime set 2
    uint32_t scale, scale_s; // N^-1 2^32 mod p, Shoup companion
    int rows;                // n d dh 2
};
struct CrtBrArgs {
    const uint32_t* key;
    Chan ch;
    const int32_t* acc_in;   // [count][2][N] torus values mod Q_CRT
    const int32_t* rot;      // [count][n] rotation amounts
    int32_t* acc_out;        // [count][2][N]
    int64_t tao_u[kCrtD], tao_u_inv[kCrtD], z[kCrtD], q_crt;
    int count, n;
};
size_t crt_br_smem_bytes(int N, int n);
int set_crt_twiddle_heads(int logN, const uint2* heads);
int launch_crt_keyconv(int logN, const CrtKeyConvArgs& a, void* stream);
int launch_crt_blind_rotate(int logN, const CrtBrArgs& a, int grid, void* stream);
int crt_blind_rotate_ctas_per_sm(int logN, int n, int* out);
int launch_draw(const DrawArgs& a, void* stream);
int launch_encrypt_lwe(const EncryptArgs& a, void* stream);

struct KeygenKskArgs {
    const int32_t* lwe_s;     // [n] 0/1
    const int32_t* rlwe_s;    // [kN] 0/1
    const int32_t* mask;      // [kN][t][n]
    const int32_t* noise;     // [kN][t]
    int32_t* ksk;             // [kN][t][n+1]
    int n, kN, t, ks_radix_bits;
};

// The lazy ("OURS") blind rotation of blindRotateLazyPipeAltNtt with its extraction, one
// ciphertext per CTA of N/2 threads, k = 1.  The key stays as the reference keeps it: the
// half TRGSW rows in the coefficient domain (torus words) and the NTT-domain s2 key; every
// CMux step rebuilds the rows of its TRGSW for the ciphertext from them.
constexpr int kLazyMaxLevels = 8;  // levels of the half rows (l_approx) and of the s2 key
// One lazy key as the kernel reads it (see LazyBrArgs).
struct LazyKeyRef {
    const void* cprime;
    const uint64_t* s2;
    const uint64_t* s2p;
};

struct LazyBrArgs {
    const int32_t* lwe_in;   // [count][n+1]
    const int64_t* lut;      // [N] test polynomial v (torus, sign-extended)
    const void* cprime;      // [n][L][2][N] half rows (a, b): int32 words at T = 32, int64 at T = 56
    const uint64_t* s2;      // [Ls][2][N] NTT-domain s2 key mod q
    const uint64_t* s2p;     // [Ls][2][N] floor(s2 2^64 / q)
    // many keys in one launch: ciphertext c uses keys[key_of[c]] (cprime, s2, s2p above
    // unused) and lut_table[lut_of[c]]; null = the single key / LUT above
    const LazyKeyRef* keys;
    const int32_t* key_of;
    const int64_t* const* lut_table;
    const int32_t* lut_of;
    const uint64_t* wf;      // [N] psi^brv(k) mod q, and Shoup companions
    const uint64_t* wfp;
    const uint64_t* wi;      // [N] psi^-brv(k) mod q, and Shoup companions
    const uint64_t* wip;
    uint64_t q;
    uint64_t qinv;           // q^-1 mod 2^64 (Montgomery products)
    uint64_t post, postp;    // N^-1 2^64 mod q and its Shoup companion
    uint64_t recomp[kLazyMaxLevels];   // 2^(T - (l'+1) radix) as a torus value, lifted mod q
    uint64_t recompp[kLazyMaxLevels];  // Shoup companions
    int32_t* big_out;        // [count][N + 1] extracted LWE, or null
    int64_t* acc_out;        // [count][2 N] accumulator, or null
    int count, n, N, L, Ls, radix_bits, torus_bits;
};
// Shared memory of one CTA: Ls + 3 polynomials of transform words (a level's batch), the
// accumulator and the mod-2N input (193 KB at N = 2048, T = 32, Ls = 8).
__host__ __device__ inline size_t lazy_br_smem_bytes(int N, int torus_bits, int n, int L, int Ls) {
    (void)L;
    size_t b = (size_t)(Ls + 3) * N * 8;
    b += 2 * (size_t)N * (torus_bits == 32 ? 4 : 8);
    b += ((size_t)n + 1) * 2;
    return (b + 15) & ~(size_t)15;
}

// The blind rotation of the group-g key family (blindRotateNtt: group 1 = blindRotateNormalNtt,
// groups 2 and 3 = blindRotateGroup2Ntt / blindRotateGroup3Ntt) with its extraction, one
// ciphertext per CTA of N/2 threads, k = 1.  The key is the reference's NTT-domain TrgswDft
// words of the levels the external product uses.
constexpr int kGroupMaxLevels = 8;  // levels of the key's decomposition (the reference's l)
struct GroupBrArgs {
    const int32_t* lwe_in;   // [count][n+1], or null when scaled_in is given
    const int32_t* scaled_in;// [count][n] mask already switched to mod 2N (with acc_in), or null
    const int64_t* lut;      // [N] test polynomial v, or null when acc_in is given
    const int64_t* acc_in;   // [count][2 N] starting accumulator, or null
    const uint64_t* key;     // [keys][L][2][2][N] NTT-domain words mod q ([lvl][col][col2])
    const uint64_t* psi_m;   // [2 N] psi^j 2^64 mod q: slot s of NTT(X^r) is psi^(r e_s)
    const uint64_t* slot_exp;// [N] e_s (odd, < 2N)
    const uint64_t* wf;      // [N] psi^brv(k) mod q, and Shoup companions
    const uint64_t* wfp;
    const uint64_t* wi;      // [N] psi^-brv(k) mod q, and Shoup companions
    const uint64_t* wip;
    uint64_t q, qinv, post, postp;  // as in LazyBrArgs
    int32_t* big_out;        // [count][N + 1] extracted LWE, or null
    int64_t* acc_out;        // [count][2 N] accumulator, or null
    int count, n, N, L, l_full, group, radix_bits, torus_bits;
};
__host__ __device__ inline size_t group_br_smem_bytes(int N, int torus_bits, int n, int L) {
    size_t b = (size_t)2 * L * N * 8;
    b += 2 * (size_t)N * (torus_bits == 32 ? 4 : 8);
    b += ((size_t)n + 1) * 2;
    return (b + 15) & ~(size_t)15;
}

// u32 words of one (step, level, row, channel) block of the device key: 2 output polys.
__host__ __device__ inline size_t key_block_words(int N) { return 2 * (size_t)N; }
__host__ __device__ inline size_t key_words(int n, int L, int N) {
    return (size_t)n * L * 2 * kChannels * key_block_words(N);
}

// Shared memory of one ciphertext slice of the blind-rotation kernel: per channel two
// padded (N + N/32)-word regions, the accumulator, int16 digits, the mod-2N input.
// Rows of the accumulator whose digits are held at once (the digit buffer is
// digit_rows x l x N int16).
__host__ __device__ constexpr int digit_rows(int torus_bits) { return torus_bits == 32 ? 2 : 1; }

// Work split of one ciphertext (blind_rotate_kernel): a team of threads per RNS channel,
// or per channel and accumulator row.
constexpr int kLayoutChannel = 0;
constexpr int kLayoutChannelRow = 1;
// A cluster of two CTAs per ciphertext, CTA h owning accumulator row h, one warp per (RNS
// channel, digit level): the levels' transforms run side by side (T = 32, N = 1024, l <= 4).
constexpr int kLayoutRowCluster = 2;
constexpr int kClusterMaxLevels = 4;

// At T = 32 each slice also keeps the first-stage product table of its forward transforms:
// psi_c^(N/2) d mod p_c for the digits d in [-64, 64] (radices up to 7), per channel.
constexpr int kTab0Half = 64;
constexpr int kTab0Words = 2 * kTab0Half + 4;  // 129 used
constexpr int kTab0Tables = 5;                 // T1, T2, T12, T3, T13 per channel (ntt.cuh, TAB = 2)
// Shared memory of one CTA of the row-cluster layout (N = 1024, T = 32): per team (channel,
// level) a padded transpose region (also its partial sum after the products) and two
// exchange regions the partner CTA writes into, the accumulator row, its digits, the mod-2N
// input, the first-stage digit tables and, for l <= kClusterStageLevels, the stage the next
// step's key rows are copied into by TMA ([l][2 rows][3 channels][1024] words) with its
// mbarrier and status word.
constexpr int kClusterStageLevels = 3;
__host__ __device__ inline size_t brc_stage_offset(int n, int L) {
    const size_t N = 1024, tbuf = N + N / 32;
    size_t b = (size_t)kChannels * L * 3 * tbuf * 4;  // transposes / partials, 2 exchange buffers
    b += N * 4 + (size_t)L * N * 2 + ((size_t)n + 1) * 2;
    b = ((b + 3) & ~(size_t)3) + (size_t)kChannels * 132 * 4;
    return (b + 127) & ~(size_t)127;
}
__host__ __device__ inline size_t brc_smem_bytes(int n, int L) {
    const size_t stage = L <= kClusterStageLevels ? (size_t)L * 2 * kChannels * 1024 * 4 : 0;
    return brc_stage_offset(n, L) + stage + 16;
}
// A cluster of six CTAs per ciphertext, CTA (h, c) owning accumulator row h in RNS channel c,
// one warp per digit level (T = 32, N = 1024, l <= 4): the latency shape with at most one
// transform warp per scheduler.
constexpr int kLayoutChannelCluster = 3;
constexpr int kCluster6Warps = 8;  // warps 0..l-1 transform; all of them decompose and recombine
// Shared memory of one CTA of the channel-cluster layout: per level a padded transpose region;
// the sum of the levels' partial products; two buffers of per-level exchange regions the
// partner CTA (the other row, the same channel) stores its transforms into; two buffers of
// the row's residues by channel after the inverse transform (two channels stored by the other
// CTAs of the row); the accumulator row, its digits, the mod-2N input, the channel's
// first-stage digit table; the stage the next step's key rows are copied into by TMA
// ([l][2 rows][1024] words); the mbarriers (the stage's, [2][kClusterMaxLevels] exchange
// regions', [2] inboxes') and a status word in 128 bytes; two buffers of per-level send
// buffers the transforms are copied to the partner from.
constexpr int kCluster6Bars = 1 + 2 * kClusterMaxLevels + 2;
__host__ __device__ inline size_t brc6_stage_offset(int n, int L) {
    const size_t N = 1024, tbuf = N + N / 32;
    size_t b = (size_t)L * tbuf * 4 + N * 4 + 2 * (size_t)L * N * 4 + 2 * 3 * N * 4;
    b += N * 4 + (size_t)L * N * 2 + ((size_t)n + 1) * 2;
    b = ((b + 3) & ~(size_t)3) + 132 * 4;
    return (b + 127) & ~(size_t)127;
}
__host__ __device__ inline size_t brc6_bars_offset(int n, int L) { return brc6_stage_offset(n, L) + (size_t)L * 2 * 1024 * 4; }
static_assert(8 * kCluster6Bars + 4 <= 128, "the barriers and the status word fit the 128 bytes before the send buffers");
__host__ __device__ inline size_t brc6_send_offset(int n, int L) { return brc6_bars_offset(n, L) + 128; }
__host__ __device__ inline size_t brc6_smem_bytes(int n, int L) { return brc6_send_offset(n, L) + (size_t)2 * L * 1024 * 4; }
__host__ __device__ inline size_t br_smem_bytes(int logN, int torus_bits, int n, int L, int layout) {
    const size_t N = (size_t)1 << logN;
    const size_t tbuf = N + N / 32;
    size_t b = kChannels * 2 * tbuf * 4;
    b += 2 * N * (torus_bits == 32 ? 4 : 8);
    b += (size_t)(layout == kLayoutChannelRow ? 2 : digit_rows(torus_bits)) * L * N * 2;
    b += ((size_t)n + 1) * 2;
    if (torus_bits == 32) b = ((b + 3) & ~(size_t)3) + (size_t)kChannels * kTab0Tables * kTab0Words * 4;
    return (b + 15) & ~(size_t)15;
}
// Uploads the first 32 forward and inverse twiddles of each channel of prime set ps
// ([3][2][32] pairs) to the constant bank of the current device.
int set_twiddle_heads(int logN, int ps, const uint2* heads);
int launch_keyconv(int logN, int ps, const KeyConvArgs& a, void* stream);
int launch_key_intt(const KeyInttArgs& a, void* stream);
int launch_wwl24_expand(const WwlExpandArgs& a, void* stream);
int launch_keygen_bsk(const KeygenBskArgs& a, void* stream);
int launch_keygen_ksk(const KeygenKskArgs& a, void* stream);
int launch_blind_rotate(int logN, int torus_bits, const BrArgs& a, void* stream);
// Resident blind-rotation CTAs per SM for these parameters and ciphertexts per CTA
// (occupancy calculator; 0 if a CTA does not fit), kNoVariant if no such kernel is compiled,
// -1 on a CUDA error.
constexpr int kNoVariant = -2;
int br_ctas_per_sm(int logN, int torus_bits, int n, int L, int per_cta, int layout);
// Six-CTA clusters of the channel-cluster layout the device runs at once (0: unknown).
int cluster6_max_clusters(int n, int L);
int launch_keyswitch(const KsArgs& a, void* stream);
// Bounded device-side waits on the current device that gave up since the library was loaded
// (the kernels then read from global memory instead); 0 on success.
int read_wait_timeouts(unsigned long long* out);
// Loads the key-switching kernel on the current device (the CUDA driver loads kernels lazily, on
// first use); 0 on success.
int preload_keyswitch();
int launch_lazy_blind_rotate(const LazyBrArgs& a, void* stream);
int launch_group_blind_rotate(const GroupBrArgs& a, void* stream);

}  // namespace yg
