// sampling.cu -- randomness drawn on the GPU, and LWE encryption.
//
// The reference draws every random value from one sequential ChaCha20 stream per thread
// (yatfhe/src/csprng.cpp), seeded from the OS; a GPU cannot replay that stream in parallel,
// so the values drawn here have the reference's distributions, not its words:
//   binary secrets (genTlweKey / genTrlweKey, yatfhe/src/tlwe.cpp:10-18, trlwe.cpp:70-81),
//   TUniform(b) noise (genTUniformNoise, yatfhe/src/numeric.cpp:47-60: b + 2 uniform bits c,
//       (c >> 1) + (c & 1) - 2^b, so the end points have probability 2^-(b+2)),
//   uniform 32-bit torus words (uniformTorusDistrib over [LWE_MIN, LWE_MAX]),
//   uniform words mod q (the NTT-domain masks of encryptTrgswMPNtt, yatfhe/src/trgsw.cpp:36-51).
// Bit-exact results against the reference go through the *_from_samples entry points, which
// take the reference's draws.
//
// Generator: the ChaCha20 block function (RFC 8439: 20 rounds of the quarter round on the
// 4 x 4 state "expand 32-byte k" | key | counter | nonce) used as a counter-mode stream:
// key = (seed, domain, 0..), nonce = (stream, 0, 0), block counter = the block index, so
// every 64-byte block is computed independently by one thread.  A domain word separates the
// arrays of one draw (secrets, BSK noise, BSK masks, ...).
#include <cuda_runtime.h>

#include <cstdint>

#include "pbs_kernels.cuh"

namespace yg {

namespace {

__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

__device__ __forceinline__ void quarter(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
    a += b;
    d = rotl32(d ^ a, 16);
    c += d;
    b = rotl32(b ^ c, 12);
    a += b;
    d = rotl32(d ^ a, 8);
    c += d;
    b = rotl32(b ^ c, 7);
}

// One 64-byte ChaCha20 block of (key, counter, nonce) into w[16].
__device__ void chacha_block(const uint32_t (&key)[8], uint32_t counter, uint32_t n0, uint32_t n1, uint32_t n2,
                             uint32_t (&w)[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                      key[4],      key[5],      key[6],      key[7],      counter, n0,     n1,     n2};
#pragma unroll
    for (int i = 0; i < 16; ++i) w[i] = s[i];
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        quarter(w[0], w[4], w[8], w[12]);
        quarter(w[1], w[5], w[9], w[13]);
        quarter(w[2], w[6], w[10], w[14]);
        quarter(w[3], w[7], w[11], w[15]);
        quarter(w[0], w[5], w[10], w[15]);
        quarter(w[1], w[6], w[11], w[12]);
        quarter(w[2], w[7], w[8], w[13]);
        quarter(w[3], w[4], w[9], w[14]);
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) w[i] += s[i];
}

__device__ __forceinline__ int64_t tuniform(uint64_t bits, int b) {
    const uint64_t mask = b + 2 >= 64 ? ~0ull : ((1ull << (b + 2)) - 1);
    const uint64_t c = bits & mask;
    return (int64_t)((c >> 1) + (c & 1)) - ((int64_t)1 << b);
}

// floor(r q / 2^128) for a uniform 128-bit r = (hi, lo): uniform on [0, q) up to 2^-67
__device__ __forceinline__ uint64_t mod_q_128(uint64_t hi, uint64_t lo, uint64_t q) {
    const uint64_t h1 = __umul64hi(hi, q), l1 = hi * q;  // hi q = h1 2^64 + l1
    const uint64_t h2 = __umul64hi(lo, q);              // (lo q) >> 64
    const uint64_t s = l1 + h2;
    return h1 + (s < l1 ? 1 : 0);
}

__global__ void draw_kernel(const DrawArgs a) {
    const uint64_t blocks = (a.count + a.per_block - 1) / a.per_block;
    for (uint64_t blk = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; blk < blocks;
         blk += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t w[16];
        const uint32_t key[8] = {(uint32_t)a.seed, (uint32_t)(a.seed >> 32), a.domain, 0, 0, 0, 0, 0};
        chacha_block(key, (uint32_t)blk, a.stream, (uint32_t)(blk >> 32), 0, w);
        const uint64_t first = blk * a.per_block;
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            if (e >= a.per_block) break;
            const uint64_t idx = first + e;
            if (idx >= a.count) break;
            switch (a.kind) {
                case kDrawBit: a.out_i32[idx] = (int32_t)(w[e] & 1); break;
                case kDrawU32: a.out_i32[idx] = (int32_t)w[e]; break;
                case kDrawTUniform: {
                    const uint64_t bits = ((uint64_t)w[2 * e + 1] << 32) | w[2 * e];
                    a.out_i32[idx] = (int32_t)tuniform(bits, a.b);
                    break;
                }
                default: {  // kDrawModQ
                    const uint64_t hi = ((uint64_t)w[4 * e + 1] << 32) | w[4 * e];
                    const uint64_t lo = ((uint64_t)w[4 * e + 3] << 32) | w[4 * e + 2];
                    a.out_u64[idx] = mod_q_128(hi, lo, a.q);
                }
            }
        }
    }
}

constexpr int kEncWarps = 8;           // warps (ciphertexts) per CTA
constexpr int kEncChunk = 32 * 16;      // mask words one warp draws per pass: a block per lane

// symEncTlwe (yatfhe/src/tlwe.cpp:21-31), one warp per ciphertext: b = sum a_i s_i + mu + e
// mod LWE_Q = 2^32.  DRAWN: the masks and the TUniform(noise_b) noise are drawn here (the
// masks of ciphertext c are words of stream 2 c + 0, its noise stream 2 c + 1 of the call's
// domain); a pass gives each lane one 16-word block, and the words go through shared memory
// (index rotated by lane / 2 so that neither the block writes nor the row reads conflict on a
// bank) so that the ciphertext row is written, and the secret read, with consecutive lanes on
// consecutive words.  Otherwise the masks and noise are read from mask / noise (streamed:
// read once), several loads in flight per lane.
template <bool DRAWN>
__global__ void __launch_bounds__(kEncWarps * 32) encrypt_lwe_kernel(const EncryptArgs a) {
    __shared__ uint32_t stage[DRAWN ? kEncWarps : 1][DRAWN ? kEncChunk : 1];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int warp = blockIdx.x * kEncWarps + wib;
    if (warp >= a.count) return;  // whole warps leave; only __syncwarp below
    const int n = a.n;
    int32_t* __restrict__ out = a.out + (size_t)warp * (n + 1);
    const int32_t* __restrict__ s = a.s;
    uint32_t sum = 0;
    const uint32_t key[8] = {(uint32_t)a.seed, (uint32_t)(a.seed >> 32), a.domain, 0, 0, 0, 0, 0};
    if constexpr (DRAWN) {
        uint32_t* st = stage[wib];
        for (int base = 0; base < n; base += kEncChunk) {
            uint32_t w[16];
            chacha_block(key, (uint32_t)(base / 16 + lane), 2u * (uint32_t)warp, (uint32_t)a.call, 0, w);
#pragma unroll
            for (int e = 0; e < 16; ++e) st[lane * 16 + ((e + (lane >> 1)) & 15)] = w[e];
            __syncwarp();
            const int lim = min(kEncChunk, n - base);
            for (int j = lane; j < lim; j += 32) {
                const int blk = j >> 4;
                const uint32_t ai = st[blk * 16 + (((j & 15) + (blk >> 1)) & 15)];
                __stcs(out + base + j, (int32_t)ai);
                sum += s[base + j] ? ai : 0u;
            }
            __syncwarp();
        }
    } else {
        const int32_t* __restrict__ mrow = a.mask + (size_t)warp * n;
#pragma unroll 8
        for (int j = lane; j < n; j += 32) {
            const uint32_t ai = (uint32_t)__ldcs(mrow + j);
            __stcs(out + j, (int32_t)ai);
            sum += s[j] ? ai : 0u;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) {
        int64_t e;
        if constexpr (DRAWN) {
            uint32_t w[16];
            chacha_block(key, 0, 2u * (uint32_t)warp + 1, (uint32_t)a.call, 0, w);
            e = tuniform(((uint64_t)w[1] << 32) | w[0], a.noise_b);
        } else {
            e = a.noise[warp];
        }
        out[n] = (int32_t)((uint32_t)a.mu[warp] + (uint32_t)e + sum);
    }
}

}  // namespace

int launch_draw(const DrawArgs& a, void* stream) {
    if (a.count == 0) return 0;
    if (a.per_block < 1 || a.per_block > 16) return -1;
    const uint64_t blocks = (a.count + a.per_block - 1) / a.per_block;
    const int threads = 256;
    const uint64_t grid = (blocks + threads - 1) / threads;
    draw_kernel<<<(unsigned)(grid < 65535 * 16 ? grid : 65535 * 16), threads, 0, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_encrypt_lwe(const EncryptArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    const unsigned grid = (unsigned)((a.count + kEncWarps - 1) / kEncWarps);
    if ((a.mask == nullptr) != (a.noise == nullptr)) return -1;  // both drawn or both given
    if (a.mask)
        encrypt_lwe_kernel<false><<<grid, kEncWarps * 32, 0, (cudaStream_t)stream>>>(a);
    else
        encrypt_lwe_kernel<true><<<grid, kEncWarps * 32, 0, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yg
