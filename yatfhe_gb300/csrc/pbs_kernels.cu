// pbs_kernels.cu -- GB300 kernels of the GINX/MP21 programmable bootstrap.
//
//   key_intt_kernel      NTT-domain key words mod q -> centred coefficient residues in the
//                        three RNS channels (done once per key upload)
//   keyconv_kernel       BSK coefficient residues -> per-channel NTT, slot layout, Montgomery
//                        form with N^-1 folded in (done once per key upload)
//   blind_rotate_kernel  rescaleTlweToNewMod + genNoiselessTrlweSample + the MP21 CMux loop
//                        (yatfhe/src/blind_rotate.cpp:1538-1565) + extractTlweFromTrlwe
//                        (yatfhe/src/trlwe.cpp:240-250); one slice of threads per
//                        ciphertext, its accumulator resident in shared memory for all n
//                        steps
//   keyswitch_kernel     switchKeyForTlwe (yatfhe/src/keyswitching.cpp:48-72) for a tile of
//                        ciphertexts x output columns, KSK rows streamed once per tile
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "ntt.cuh"
#include "pbs_kernels.cuh"

namespace yg {

// Bounded device-side waits that gave up (the kernel then took its fallback path).
__device__ unsigned long long g_wait_timeouts;

namespace {

__device__ __forceinline__ Chan pick_chan(const Chan (&c)[kChannels], int team) {
    return team == 0 ? c[0] : (team == 1 ? c[1] : c[2]);
}

// L2 policy for bootstrapping-key reads: every ciphertext of a launch re-reads the whole
// key, so its lines are kept in L2 ahead of the streamed inputs and outputs.
__device__ __forceinline__ uint64_t l2_evict_last_policy() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ uint4 ldg_keep(const uint4* p, uint64_t pol) {
    uint4 v;
    asm("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(p), "l"(pol));
    return v;
}

// Bulk copies into shared memory (TMA, cp.async.bulk) tracked by an mbarrier: one thread
// arms the barrier with the byte count and issues the copies; consumers wait for the phase.
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// global -> this CTA's shared memory, `bytes` (a multiple of 16) from 16-byte aligned addresses
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// Waits for the barrier phase of this parity to complete, for at most `cycles` clocks
// (false: it gave up).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long cycles) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > cycles) return false;
    }
}
// about one second at the GB300's clock: far beyond any copy's latency
constexpr long long kWaitCycles = 2000000000LL;

// zeroMeanDigits (yatfhe/include/yatfhe/gadget_decomposition.h:76-95): signed balanced
// digits of the top L*radix bits of a W-bit value, rounded half away from zero, carry
// propagated from the least significant level, ties broken by the top bit of the next
// window; digit(level) for level 0 = most significant.
template <typename U, int W, typename Emit>
__device__ __forceinline__ void zero_mean_digits(U u, int L, int radix, Emit&& emit) {
    constexpr U wmask = (W >= (int)(8 * sizeof(U))) ? ~U(0) : ((U(1) << W) - 1);
    u &= wmask;
    const bool neg = (u >> (W - 1)) & 1;
    const int dropped = W - L * radix;
    const U bias = dropped > 0 ? (U(1) << (dropped - 1)) : U(0);
    const U m = (neg ? (U(0) - u) & wmask : u) + bias;
    const int B = 1 << radix, halfB = B >> 1;
    int carry = 0;
    for (int level = L - 1; level >= 0; --level) {
        const int shift = W - (level + 1) * radix;
        const int digit = (int)((m >> shift) & (U)(B - 1)) + carry;
        const int tie = level > 0 ? (int)((m >> (shift + 2 * radix - 1)) & 1) : 0;
        carry = (digit > halfB) | ((digit == halfB) & tie);
        const int bal = carry ? digit - B : digit;
        emit(level, neg ? -bal : bal);
    }
}

// modSwitchFromTorusGeneral (yatfhe/src/numeric.cpp:189-208) downscaling by 2^sh with a
// power-of-two target of `bits` bits: round half away from zero, then sign-extend.
__device__ __forceinline__ int64_t modswitch_down(int64_t x, int sh, int bits) {
    const int64_t h = (int64_t)1 << (sh - 1);
    const int64_t r = x >= 0 ? ((x + h) >> sh) : -((-x + h) >> sh);
    return (int64_t)((uint64_t)r << (64 - bits)) >> (64 - bits);
}

template <int T>
struct TorusOf;
template <>
struct TorusOf<32> {
    using type = int32_t;
    using utype = uint32_t;
};
template <>
struct TorusOf<56> {
    using type = int64_t;
    using utype = uint64_t;
};

// torus a - b reduced to T bits (int32 wrap for T = 32, longModPow2 for T = 56).
template <int T>
__device__ __forceinline__ typename TorusOf<T>::type tsub(typename TorusOf<T>::type a, typename TorusOf<T>::type b) {
    using U = typename TorusOf<T>::utype;
    if constexpr (T == 32) return (int32_t)((U)a - (U)b);
    else return sext<56>((int64_t)((U)a - (U)b));
}

template <int T>
__device__ __forceinline__ typename TorusOf<T>::type tneg(typename TorusOf<T>::type a) {
    using U = typename TorusOf<T>::utype;
    if constexpr (T == 32) return (int32_t)(U(0) - (U)a);
    else return sext<56>((int64_t)(U(0) - (U)a));
}

template <int LOGN, int PS>
__global__ void __launch_bounds__(3 * TeamShape<LOGN>::S) keyconv_kernel(const KeyConvArgs a) {
    using Sh = TeamShape<LOGN>;
    constexpr int N = Sh::N, S = Sh::S;
    __shared__ uint32_t tb[kChannels * Sh::TBUF];
    const int poly = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int team = warp / Sh::WARPS;
    const int tt = (warp % Sh::WARPS) * 32 + lane;
    const Chan ch = pick_chan(a.ch, team);
    const uint32_t sc = team == 0 ? a.scale[0] : (team == 1 ? a.scale[1] : a.scale[2]);
    const uint32_t scs = team == 0 ? a.scale_s[0] : (team == 1 ? a.scale_s[1] : a.scale_s[2]);
    const uint32_t* src = a.residues + ((size_t)poly * kChannels + team) * N;
    uint32_t x[32];
    const uint32_t bias = fwd_bias_residues<LOGN, PS>(ch.p);
#pragma unroll
    for (int r = 0; r < 32; ++r) x[r] = src[r * S + tt] + bias;
    ntt_forward<LOGN, PS>(x, tb + team * Sh::TBUF, tt, team, team, ch);
    const int blk = poly >> 1, o = poly & 1;
    uint32_t* dst = a.key + ((size_t)blk * kChannels + team) * key_block_words(N);
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        const uint32_t y = reduce_once(reduce_once(mulshoup(x[r], sc, scs, ch.p), ch.two_p), ch.p);
        dst[((o * 8 + (r >> 2)) * S + tt) * 4 + (r & 3)] = y;
    }
}

// x w mod q for x < q < 2^63, w < q, wp = floor(w 2^64 / q) (Shoup).
__device__ __forceinline__ uint64_t mulshoup64(uint64_t x, uint64_t w, uint64_t wp, uint64_t q) {
    const uint64_t qh = __umul64hi(x, wp);
    const uint64_t r = x * w - qh * q;
    return r >= q ? r - q : r;
}

// Inverse negacyclic transform mod q of the N words in shared memory, without the N^-1
// factor: Gentleman-Sande, stage with butterfly span t pairs (2 i t + j, 2 i t + j + t)
// with twiddle w[N / (2t) + i] = psi^-brv(N / (2t) + i); bit-reversed slots in, natural
// coefficients out.  All threads of the block take part; ends synchronised.
__device__ void q_inverse_in_smem(uint64_t* sw, int N, const uint64_t* w, const uint64_t* wp, uint64_t q) {
    for (int t = 1; t < N; t <<= 1) {
        const int h = N / (2 * t);
        for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
            const int i = b / t, j = b - i * t;
            const int xi = 2 * i * t + j, yi = xi + t;
            const uint64_t u = sw[xi], v = sw[yi];
            const uint64_t s = u + v;
            sw[xi] = s >= q ? s - q : s;
            sw[yi] = mulshoup64(u >= v ? u - v : u + q - v, w[h + i], wp[h + i], q);
        }
        __syncthreads();
    }
}

// Forward negacyclic transform mod q in shared memory, the exact inverse of the above:
// Cooley-Tukey, stage m (= 1, 2, .., N/2) with span t = N / (2m) pairs (2 i t + j,
// 2 i t + j + t) with twiddle w[m + i] = psi^brv(m + i); natural coefficients in,
// bit-reversed slots out (the transform HEXL's ComputeForward documents).  Ends synchronised.
__device__ void q_forward_in_smem(uint64_t* sw, int N, const uint64_t* w, const uint64_t* wp, uint64_t q) {
    for (int m = 1, t = N / 2; m < N; m <<= 1, t >>= 1) {
        for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
            const int i = b / t, j = b - i * t;
            const int xi = 2 * i * t + j, yi = xi + t;
            const uint64_t u = sw[xi], v = mulshoup64(sw[yi], w[m + i], wp[m + i], q);
            const uint64_t s = u + v;
            sw[xi] = s >= q ? s - q : s;
            sw[yi] = u >= v ? u - v : u + q - v;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) key_intt_kernel(const KeyInttArgs a) {
    extern __shared__ uint64_t sw[];  // [N]
    const int N = a.N, poly = blockIdx.x;
    const uint64_t q = a.q;
    const uint64_t* src = a.words + (size_t)poly * N;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const uint64_t v = src[j];
        if (v >= q) atomicExch(a.bad, 1);
        sw[j] = v < q ? v : 0;
    }
    __syncthreads();
    q_inverse_in_smem(sw, N, a.w, a.wp, q);
    const uint64_t half = (q + 1) / 2;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const uint64_t v = mulshoup64(sw[j], a.ninv, a.ninvp, q);
        for (int c = 0; c < kChannels; ++c) {
            const uint64_t p = a.p[c];
            // centred representative: v >= (q+1)/2 stands for v - q
            a.residues[((size_t)poly * kChannels + c) * N + j] =
                v >= half ? (uint32_t)((p - (q - v) % p) % p) : (uint32_t)(v % p);
        }
    }
}

// switchTrlweToSecretEmbeddingNtt (yatfhe/src/trgsw.cpp:861-905) for one (key index i,
// level lvl) per block, k = 1: the mask of cPrime[lvl] back to the torus (applyIntt,
// ntt_hexl.cpp:153-175: inverse transform, centred mod q, low T bits), its zero-mean digits
// (decomposeRow), and per digit level l' one forward transform and the products with the s2
// key: c.a = sum NTT(d_l') . s2[l'].a + cPrime.b, c.b = sum NTT(d_l') . s2[l'].b (mod q).
// Writes the GINX level [c (a, b) | cPrime (a, b)] in the layout of the NTT-domain BSK.
// N / 2 threads; thread t owns coefficients / slots t and t + N / 2 outside the transforms.
template <int T>
__global__ void __launch_bounds__(1024) wwl24_expand_kernel(const WwlExpandArgs a) {
    using U = typename TorusOf<T>::utype;
    extern __shared__ uint64_t sw[];  // [N]
    const int N = a.N, H = N / 2, t = threadIdx.x;
    const int i = blockIdx.x / a.L, lvl = blockIdx.x - i * a.L;
    const uint64_t q = a.q;
    const size_t row = 2 * (size_t)N;
    const uint64_t* cp = a.cprime + ((size_t)i * a.L + lvl) * row;  // [a | b]
    uint64_t* g = a.out + ((size_t)i * a.L + lvl) * 2 * row;         // [c: a | b][cPrime: a | b]
    uint64_t own[2][2];  // this thread's cPrime words: [coefficient e][a, b]
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const int j = t + e * H;
#pragma unroll
        for (int poly = 0; poly < 2; ++poly) {
            const uint64_t v = cp[poly * N + j];
            if (v >= q) atomicExch(a.bad, 1);
            own[e][poly] = v < q ? v : 0;
            g[row + poly * N + j] = own[e][poly];
        }
        sw[j] = own[e][0];
    }
    __syncthreads();
    q_inverse_in_smem(sw, N, a.wi, a.wip, q);
    int dg[2][kWwlMaxLevels];
    const uint64_t half = (q + 1) / 2;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const uint64_t v = mulshoup64(sw[t + e * H], a.ninv, a.ninvp, q);
        const int64_t centred = v >= half ? (int64_t)(v - q) : (int64_t)v;
        zero_mean_digits<U, T>((U)sext<T>(centred), a.Ls, a.radix_bits, [&](int level, int d) {
#pragma unroll
            for (int x = 0; x < kWwlMaxLevels; ++x)
                if (x == level) dg[e][x] = d;
        });
    }
    uint64_t acc[2][2] = {{0, 0}, {0, 0}};  // [coefficient e][a, b]
#pragma unroll
    for (int lv = 0; lv < kWwlMaxLevels; ++lv) {
        if (lv >= a.Ls) break;
        __syncthreads();  // the previous transform's slots have been read
#pragma unroll
        for (int e = 0; e < 2; ++e) sw[t + e * H] = dg[e][lv] < 0 ? q - (uint64_t)(-dg[e][lv]) : (uint64_t)dg[e][lv];
        __syncthreads();
        q_forward_in_smem(sw, N, a.wf, a.wfp, q);
        const size_t s2o = (size_t)lv * row;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int j = t + e * H;
            const uint64_t D = sw[j];
#pragma unroll
            for (int poly = 0; poly < 2; ++poly) {
                const uint64_t m = mulshoup64(D, a.s2[s2o + poly * N + j], a.s2p[s2o + poly * N + j], q);
                const uint64_t s = acc[e][poly] + m;
                acc[e][poly] = s >= q ? s - q : s;
            }
        }
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const int j = t + e * H;
        const uint64_t s = acc[e][0] + own[e][1];  // c.a += cPrime.b
        g[j] = s >= q ? s - q : s;
        g[N + j] = acc[e][1];
    }
}

// encryptTrgswMPNtt's samples (yatfhe/src/trgsw.cpp:36-51 with symEncTrlweNttSimple,
// yatfhe/src/trlwe.cpp:24-46,58-60), one per CTA: b = NTT(sext(mu + e)) + sum_r a_r . NTT(s_r)
// mod q with the mask a given in the NTT domain; the cPrime row (row k) carries
// mu = s_i 2^(T - (lvl+1) radix) at coefficient 0, row r < k carries it on its mask a_r as
// NTT(mu) (a constant polynomial: mu in every slot).
template <int T>
__global__ void __launch_bounds__(1024) keygen_bsk_kernel(const KeygenBskArgs a) {
    extern __shared__ uint64_t sw[];  // [N]
    const int N = a.N, H = N / 2, k = a.k, t = threadIdx.x;
    const int row = blockIdx.x % (k + 1);
    const int lvl = (blockIdx.x / (k + 1)) % a.L;
    const int i = blockIdx.x / ((k + 1) * a.L);
    const uint64_t q = a.q;
    const int32_t* e = a.noise + (size_t)blockIdx.x * N;
    const uint64_t* msk = a.mask + (size_t)blockIdx.x * k * N;
    uint64_t* out = a.words + (size_t)blockIdx.x * (k + 1) * N;
    const int64_t mu = sext<T>((int64_t)a.lwe_s[i] << (T - (lvl + 1) * a.radix_bits));
    const uint64_t mu_q = mu < 0 ? (uint64_t)(mu + (int64_t)q) : (uint64_t)mu;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j = t + h * H;
        const int64_t v = sext<T>((row == k && j == 0 ? mu : 0) + (int64_t)e[j]);
        sw[j] = v < 0 ? (uint64_t)(v + (int64_t)q) : (uint64_t)v;
    }
    __syncthreads();
    q_forward_in_smem(sw, N, a.wf, a.wfp, q);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j = t + h * H;
        uint64_t b = sw[j];
        for (int r = 0; r < k; ++r) {
            uint64_t m = msk[(size_t)r * N + j];
            if (m >= q) {
                atomicExch(a.bad, 1);
                m = 0;
            }
            const uint64_t prod = mulshoup64(m, a.s_ntt[(size_t)r * N + j], a.s_ntt_p[(size_t)r * N + j], q);
            b = b + prod >= q ? b + prod - q : b + prod;
            if (r == row) m = m + mu_q >= q ? m + mu_q - q : m + mu_q;  // a_r += NTT(mu) on row r
            out[(size_t)r * N + j] = m;
        }
        out[(size_t)k * N + j] = b;
    }
}

// genTlweKeySwitchingKey (yatfhe/src/keyswitching.cpp:19-29), one warp per sample:
// ksk[i][j] = (a, sum a s + s'_i 2^(32 - (j+1) ksRadix) + e) mod 2^32 (symEncTlwe,
// yatfhe/src/tlwe.cpp:21-31, whose sign extensions are the identity mod 2^32).
__global__ void __launch_bounds__(256) keygen_ksk_kernel(const KeygenKskArgs a) {
    const int sample = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (sample >= a.kN * a.t) return;  // whole warps leave together
    const int i = sample / a.t, j = sample - i * a.t;
    const int32_t* m = a.mask + (size_t)sample * a.n;
    int32_t* dst = a.ksk + (size_t)sample * (a.n + 1);
    uint32_t sum = 0;
    for (int x = lane; x < a.n; x += 32) {
        const int32_t v = m[x];
        dst[x] = v;
        if (a.lwe_s[x]) sum += (uint32_t)v;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
    if (lane == 0) {
        const uint32_t msg = (uint32_t)a.rlwe_s[i] << (32 - (j + 1) * a.ks_radix_bits);
        dst[a.n] = (int32_t)(sum + msg + (uint32_t)a.noise[sample]);
    }
}

// torus a + b reduced to T bits.
template <int T>
__device__ __forceinline__ typename TorusOf<T>::type tadd(typename TorusOf<T>::type a, typename TorusOf<T>::type b) {
    using U = typename TorusOf<T>::utype;
    if constexpr (T == 32) return (int32_t)((U)a + (U)b);
    else return sext<56>((int64_t)((U)a + (U)b));
}

// x y 2^-64 mod q for x, y < q < 2^62 (Montgomery; qinv = q^-1 mod 2^64): x y - m q with
// m = (x y) qinv mod 2^64 has zero low word, so the high words' difference is exact.
__device__ __forceinline__ uint64_t montmul64(uint64_t x, uint64_t y, uint64_t q, uint64_t qinv) {
    const uint64_t lo = x * y, hi = __umul64hi(x, y);
    const uint64_t mh = __umul64hi(lo * qinv, q);
    return hi >= mh ? hi - mh : hi + q - mh;
}

// x w mod q up to one multiple of q: x w - floor(x wp / 2^64) q is in [0, 2q) for any
// 64-bit x, w < q, wp = floor(w 2^64 / q) (Shoup without the final correction).
__device__ __forceinline__ uint64_t mulshoup64_lazy(uint64_t x, uint64_t w, uint64_t wp, uint64_t q) {
    return x * w - __umul64hi(x, wp) * q;
}

// symEncTrlweMultiSampleSimple (yatfhe/src/trlwe.cpp:40-47 initTrlweMultiSampleSimple then
// :62-64 symEncTrlweNttSimple): b = NTT(sext(mu + e)) + sum_r a_r . NTT(s_r) mod q with the
// masks a_r uniform in the NTT domain; N/2 threads, one sample per pass of a CTA.  Each CTA
// first transforms the secret into shared memory in Montgomery form (NTT(s) 2^64 mod q, from
// one Montgomery product with 2^128 mod q), so one Montgomery product with a mask gives
// a_r . NTT(s_r) mod q exactly.
template <int T>
__global__ void __launch_bounds__(1024) encrypt_rlwe_ntt_kernel(const EncryptRlweArgs a) {
    extern __shared__ uint64_t sw[];  // [N] transform, then [k][N] NTT(s) 2^64 mod q
    const int N = a.N, k = a.k;
    uint64_t* sm = sw + N;
    const uint64_t q = a.q;
    for (int r = 0; r < k; ++r) {
        for (int j = threadIdx.x; j < N; j += blockDim.x) sw[j] = a.s[(size_t)r * N + j] != 0 ? 1 : 0;
        __syncthreads();
        q_forward_in_smem(sw, N, a.wf, a.wfp, q);
        for (int j = threadIdx.x; j < N; j += blockDim.x) sm[(size_t)r * N + j] = montmul64(sw[j], a.r2, q, a.qinv);
        __syncthreads();
    }
    for (int c = blockIdx.x; c < a.count; c += gridDim.x) {
        const int64_t* mu = a.mu + (size_t)c * N;
        const int32_t* e = a.noise + (size_t)c * N;
        for (int j = threadIdx.x; j < N; j += blockDim.x) {
            const int64_t v = sext<T>(mu[j] + (int64_t)e[j]);
            sw[j] = v < 0 ? (uint64_t)(v + (int64_t)q) : (uint64_t)v;
        }
        __syncthreads();
        q_forward_in_smem(sw, N, a.wf, a.wfp, q);
        const uint64_t* msk = a.mask + (size_t)c * k * N;
        uint64_t* out = a.out + (size_t)c * (k + 1) * N;
        for (int j = threadIdx.x; j < N; j += blockDim.x) {
            uint64_t b = sw[j];
            for (int r = 0; r < k; ++r) {
                uint64_t m = msk[(size_t)r * N + j];
                if (m >= q) {
                    if (a.bad) atomicExch(a.bad, 1);
                    m = 0;
                }
                const uint64_t prod = montmul64(m, sm[(size_t)r * N + j], q, a.qinv);
                b = b + prod >= q ? b + prod - q : b + prod;
                out[(size_t)r * N + j] = m;
            }
            out[(size_t)k * N + j] = b;
        }
        __syncthreads();  // sw is rewritten by the next sample
    }
}

// M forward transforms mod q of the polynomials sw[k N .. k N + N), k < M, in the convention
// of q_forward_in_smem, sharing each stage's twiddle loads and barrier.  Harvey's lazy
// butterflies: words in [0, 4q) in and out (4q < 2^64 for both moduli), so the results are
// the transform's values up to multiples of q.  Ends synchronised.
__device__ void q_forward_batch(uint64_t* sw, int M, int N, int logN, const uint64_t* w, const uint64_t* wp,
                                uint64_t q) {
    const uint64_t q2 = 2 * q;
    // the lazy Cooley-Tukey butterfly: u reduced below 2q, v times the twiddle (Shoup, < 2q)
    auto bfly = [&](uint64_t& u, uint64_t& v, uint64_t W, uint64_t Wp) {
        const uint64_t ur = u >= q2 ? u - q2 : u;
        const uint64_t t = mulshoup64_lazy(v, W, Wp, q);
        u = ur + t;
        v = ur + q2 - t;
    };
    // blockDim.x is a multiple of N/4 (the kernels run N/2 threads): each thread keeps one group
    // index and its twiddles for a pass and steps through the M polynomials
    const int quarter = N >> 2, qshift = logN - 2;
    const int gi = threadIdx.x & (quarter - 1), k0 = threadIdx.x >> qshift, kstep = blockDim.x >> qshift;
    int s = 0;
    // two stages per pass: each thread takes groups of four words (one per butterfly of both
    // stages), the same butterflies in the same order as two radix-2 passes
    for (; s + 1 < logN; s += 2) {
        const int m = 1 << s, lt = logN - 1 - s, t = 1 << lt, t2 = t >> 1;
        const int i = gi >> (lt - 1), j = gi & (t2 - 1);
        const uint64_t Wa = w[m + i], Wap = wp[m + i];
        const uint64_t Wb = w[2 * m + 2 * i], Wbp = wp[2 * m + 2 * i];
        const uint64_t Wc = w[2 * m + 2 * i + 1], Wcp = wp[2 * m + 2 * i + 1];
        for (int k = k0; k < M; k += kstep) {
            uint64_t* p = sw + (size_t)k * N + (i << (lt + 1)) + j;
            uint64_t x0 = p[0], x1 = p[t2], x2 = p[t], x3 = p[t + t2];
            bfly(x0, x2, Wa, Wap);
            bfly(x1, x3, Wa, Wap);
            bfly(x0, x1, Wb, Wbp);
            bfly(x2, x3, Wc, Wcp);
            p[0] = x0;
            p[t2] = x1;
            p[t] = x2;
            p[t + t2] = x3;
        }
        __syncthreads();
    }
    if (s < logN) {  // an odd stage count: the last stage (span 1) alone
        const int m = 1 << s;
        const int i = threadIdx.x & ((N >> 1) - 1);
        const uint64_t W = w[m + i], Wp = wp[m + i];
        for (int k = threadIdx.x >> (logN - 1); k < M; k += blockDim.x >> (logN - 1)) {
            uint64_t* p = sw + (size_t)k * N + 2 * i;
            uint64_t x0 = p[0], x1 = p[1];
            bfly(x0, x1, W, Wp);
            p[0] = x0;
            p[1] = x1;
        }
        __syncthreads();
    }
}

// M inverse transforms mod q (the convention of q_inverse_in_smem, no N^-1), batched as above,
// with lazy butterflies on words in [0, 2q) in and out.
__device__ void q_inverse_batch(uint64_t* sw, int M, int N, int logN, const uint64_t* w, const uint64_t* wp,
                                uint64_t q) {
    const uint64_t q2 = 2 * q;
    // the lazy Gentleman-Sande butterfly
    auto bfly = [&](uint64_t& u, uint64_t& v, uint64_t W, uint64_t Wp) {
        const uint64_t sum = u + v;
        const uint64_t d = u + q2 - v;
        u = sum >= q2 ? sum - q2 : sum;
        v = mulshoup64_lazy(d, W, Wp, q);
    };
    const int quarter = N >> 2, qshift = logN - 2;
    const int gi = threadIdx.x & (quarter - 1), k0 = threadIdx.x >> qshift, kstep = blockDim.x >> qshift;
    int lt = 0;
    for (; lt + 1 < logN; lt += 2) {
        const int t = 1 << lt, h = N >> (lt + 1);
        const int i = gi >> lt, j = gi & (t - 1);
        const uint64_t Wa = w[h + 2 * i], Wap = wp[h + 2 * i];
        const uint64_t Wb = w[h + 2 * i + 1], Wbp = wp[h + 2 * i + 1];
        const uint64_t Wc = w[(h >> 1) + i], Wcp = wp[(h >> 1) + i];
        for (int k = k0; k < M; k += kstep) {
            uint64_t* p = sw + (size_t)k * N + (i << (lt + 2)) + j;
            uint64_t x0 = p[0], x1 = p[t], x2 = p[2 * t], x3 = p[3 * t];
            bfly(x0, x1, Wa, Wap);
            bfly(x2, x3, Wb, Wbp);
            bfly(x0, x2, Wc, Wcp);
            bfly(x1, x3, Wc, Wcp);
            p[0] = x0;
            p[t] = x1;
            p[2 * t] = x2;
            p[3 * t] = x3;
        }
        __syncthreads();
    }
    if (lt < logN) {  // the last stage (span N/2) alone
        const int t = 1 << lt;
        const int j = threadIdx.x & ((N >> 1) - 1);
        const uint64_t W = w[1], Wp = wp[1];
        for (int k = threadIdx.x >> (logN - 1); k < M; k += blockDim.x >> (logN - 1)) {
            uint64_t* p = sw + (size_t)k * N + j;
            uint64_t x0 = p[0], x1 = p[t];
            bfly(x0, x1, W, Wp);
            p[0] = x0;
            p[t] = x1;
        }
        __syncthreads();
    }
}

// blindRotateLazyPipeAltNtt (yatfhe/src/blind_rotate.cpp:995-1135) and the extraction, one
// ciphertext per CTA of N/2 threads; thread t owns coefficients and transform slots t and
// t + N/2.  The arithmetic is the reference's: words mod q, transformed in shared memory in
// HEXL's negacyclic convention (q_forward_batch / q_inverse_batch), products with key words
// or constants by Shoup multiplication, products of two computed words by Montgomery
// multiplication (whose 2^-64 the final N^-1 2^64 scaling removes).
//   first component: acc = X^(-b) ((X^(a_0) - 1) derived + (0, v)), derived =
//     INTT(sum_lvl NTT(digit lvl of v) . NTT(cPrime_0[lvl]))        (:1117-1124)
//   step i (a_i != 0): acc = acc [x] TRGSW_i (externalProductTrgswMPNttInPlace), where level
//     lvl of TRGSW_i comes from the rotated half row cP = (X^(a_i) - 1) cPrime_i[lvl],
//     cP.b[0] += 2^(T - (lvl+1) radix), and its mask digits D_l' (l' < Ls, transformed):
//       cPrime.a = sum D_l' . 2^(T - (l'+1) radix),  cPrime.b = NTT(cP.b),
//       c.a = sum D_l' . s2[l'].a + NTT(cP.b),       c.b = sum D_l' . s2[l'].b
//     (stageA / stageB, :1036-1085).  Per level the Ls digit polynomials, cP.b and the
//     accumulator's two digit polynomials of that level go through one batch of Ls + 3
//     transforms; the level's rows are then formed slot by slot in registers and multiplied
//     into the product at once, so nothing of TRGSW_i is stored.
template <int T>
__global__ void __launch_bounds__(1024, 1) lazy_blind_rotate_kernel(const LazyBrArgs a) {
    using TT = typename TorusOf<T>::type;
    using U = typename TorusOf<T>::utype;
    extern __shared__ __align__(16) unsigned char lz_smem[];
    const int N = a.N, H = N >> 1, t = threadIdx.x, n = a.n, L = a.L, Ls = a.Ls, rb = a.radix_bits;
    const int logN = 31 - __clz(N);
    const int ct = blockIdx.x;
    const uint64_t q = a.q, qinv = a.qinv;
    const int M = Ls + 3;
    uint64_t* sw = reinterpret_cast<uint64_t*>(lz_smem);                  // [Ls + 3][N]
    TT* acc = reinterpret_cast<TT*>(sw + (size_t)M * N);                  // [2][N]
    int16_t* sa = reinterpret_cast<int16_t*>(acc + 2 * N);                // [n + 1]
    // this ciphertext's key and test polynomial (one of many when the launch has tables)
    const LazyKeyRef kr = a.key_of ? a.keys[a.key_of[ct]] : LazyKeyRef{a.cprime, a.s2, a.s2p};
    const TT* cpr = static_cast<const TT*>(kr.cprime);
    const uint64_t* s2 = kr.s2;
    const uint64_t* s2p = kr.s2p;
    const int64_t* lut = a.lut_of ? a.lut_table[a.lut_of[ct]] : a.lut;
    const int jj[2] = {t, t + H};

    auto lift = [q](int64_t x) -> uint64_t { return x < 0 ? (uint64_t)(x + (int64_t)q) : (uint64_t)x; };
    auto addq = [q](uint64_t x, uint64_t y) -> uint64_t {
        const uint64_t s = x + y;
        return s >= q ? s - q : s;
    };
    const uint64_t q2 = 2 * q;
    // a forward transform's word (in [0, 4q)) reduced to [0, q)
    auto red4 = [q, q2](uint64_t x) -> uint64_t {
        x = x >= q2 ? x - q2 : x;
        return x >= q ? x - q : x;
    };
    // applyIntt's last steps (yatfhe/src/ntt_hexl.cpp:153-175): scale, centre, low T bits
    // (the word, in [0, 2q) after the lazy inverse transform, is reduced by the product).
    auto to_torus = [&](uint64_t v) -> TT {
        v = mulshoup64(v, a.post, a.postp, q);
        const int64_t c = v >= (q + 1) / 2 ? (int64_t)(v - q) : (int64_t)v;
        if constexpr (T == 32) return (int32_t)(uint32_t)(uint64_t)c;
        else return sext<56>(c);
    };
    // (X^r p)[j] for r in [0, 2N) (rotateTorusPolynomial, yatfhe/src/polynomial.cpp:184-193)
    auto rot_at = [N](const TT* p, int r, int j) -> TT {
        int x = j - r;
        bool neg = false;
        if (x < 0) {
            x += N;
            neg = true;
        }
        if (x < 0) {
            x += N;
            neg = false;
        }
        const TT v = p[x];
        return neg ? tneg<T>(v) : v;
    };
    auto norm = [N](int r) {
        r %= 2 * N;
        return r < 0 ? r + 2 * N : r;
    };
    // digit `lvl` of the zero-mean decomposition of x into `levels` digits
    auto digit_at = [rb](TT x, int levels, int lvl) {
        int d = 0;
        zero_mean_digits<U, T>((U)x, levels, rb, [&](int level, int v) {
            if (level == lvl) d = v;
        });
        return d;
    };
    // both accumulator polynomials from the transform slots of sw[0..2N), scaled to the torus
    auto inverse_to_acc = [&](const uint64_t (&h)[2][2]) {
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) sw[poly * N + jj[e]] = h[poly][e];
        __syncthreads();
        q_inverse_batch(sw, 2, N, logN, a.wi, a.wip, q);
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) acc[poly * N + jj[e]] = to_torus(sw[poly * N + jj[e]]);
        __syncthreads();
    };

    // rescaleTlweToNewMod into mod 2N (yatfhe/src/tlwe.cpp:75-81)
    const int32_t* in = a.lwe_in + (size_t)ct * (n + 1);
    for (int i = t; i <= n; i += H) sa[i] = (int16_t)modswitch_down(in[i], 31 - logN, logN + 1);

    // first component (deriveFirstComponentNtt, yatfhe/src/trgsw.cpp:929-955, with the digits
    // of v that prepareGdV transforms, :911-927)
    {
        uint64_t h[2][2] = {{0, 0}, {0, 0}};
        for (int lvl = 0; lvl < L; ++lvl) {
            const TT* src = cpr + (size_t)lvl * 2 * N;  // key index 0
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int j = jj[e];
                sw[j] = lift(digit_at((TT)lut[j], L, lvl));
                sw[N + j] = lift((int64_t)src[j]);
                sw[2 * N + j] = lift((int64_t)src[N + j]);
            }
            __syncthreads();
            q_forward_batch(sw, 3, N, logN, a.wf, a.wfp, q);
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int j = jj[e];
                const uint64_t V = red4(sw[j]);
                h[0][e] = addq(h[0][e], montmul64(V, red4(sw[N + j]), q, qinv));
                h[1][e] = addq(h[1][e], montmul64(V, red4(sw[2 * N + j]), q, qinv));
            }
            __syncthreads();
        }
        inverse_to_acc(h);
        TT tv[2][2];
        const int r0 = norm(sa[0]);
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int j = jj[e];
                TT x = tsub<T>(rot_at(acc + poly * N, r0, j), acc[poly * N + j]);
                if (poly == 1) x = tadd<T>(x, (TT)lut[j]);
                tv[poly][e] = x;
            }
        __syncthreads();
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) acc[poly * N + jj[e]] = tv[poly][e];
        __syncthreads();
        const int rb0 = norm(-(int)sa[n]);
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) tv[poly][e] = rot_at(acc + poly * N, rb0, jj[e]);
        __syncthreads();
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) acc[poly * N + jj[e]] = tv[poly][e];
        __syncthreads();
    }

    for (int i = 1; i < n; ++i) {
        const int ai = sa[i];
        if (ai == 0) continue;  // the same for every thread of the CTA
        const int r = norm(ai);
        uint64_t acch[2][2] = {{0, 0}, {0, 0}};
        for (int lvl = 0; lvl < L; ++lvl) {
            const TT* cp = cpr + ((size_t)i * L + lvl) * 2 * N;
            const int sh = T - (lvl + 1) * rb;
            TT one;
            if constexpr (T == 32) one = (int32_t)((uint32_t)1 << sh);
            else one = sext<56>((int64_t)1 << sh);
            // stageA (rotateTrlweMinusOneBPlusOne, then the mask's Ls digits, decomposeRow) and
            // the accumulator's digits of this level: the inputs of the level's transforms
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int j = jj[e];
                const TT ra = tsub<T>(rot_at(cp, r, j), cp[j]);
                TT rbv = tsub<T>(rot_at(cp + N, r, j), cp[N + j]);
                if (j == 0) rbv = tadd<T>(rbv, one);
                zero_mean_digits<U, T>((U)ra, Ls, rb, [&](int level, int d) { sw[(size_t)level * N + j] = lift(d); });
                sw[(size_t)Ls * N + j] = lift((int64_t)rbv);
                sw[(size_t)(Ls + 1) * N + j] = lift(digit_at(acc[j], L, lvl));
                sw[(size_t)(Ls + 2) * N + j] = lift(digit_at(acc[N + j], L, lvl));
            }
            __syncthreads();
            q_forward_batch(sw, M, N, logN, a.wf, a.wfp, q);
            // stageB slot by slot, and the level's share of the external product
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int j = jj[e];
                // sums kept in [0, 2q): lazy products of the raw [0, 4q) words
                auto add2 = [q2](uint64_t x, uint64_t y) -> uint64_t {
                    const uint64_t s = x + y;
                    return s >= q2 ? s - q2 : s;
                };
                uint64_t ca = 0, cb = 0, cpa = 0;
                for (int gl = 0; gl < Ls; ++gl) {
                    const uint64_t D = sw[(size_t)gl * N + j];
                    const size_t o = (size_t)gl * 2 * N + j;
                    ca = add2(ca, mulshoup64_lazy(D, s2[o], s2p[o], q));
                    cb = add2(cb, mulshoup64_lazy(D, s2[o + N], s2p[o + N], q));
                    cpa = add2(cpa, mulshoup64_lazy(D, a.recomp[gl], a.recompp[gl], q));
                }
                const uint64_t bh = red4(sw[(size_t)Ls * N + j]);
                ca = addq(ca >= q ? ca - q : ca, bh);
                cb = cb >= q ? cb - q : cb;
                cpa = cpa >= q ? cpa - q : cpa;
                const uint64_t xa = red4(sw[(size_t)(Ls + 1) * N + j]), xb = red4(sw[(size_t)(Ls + 2) * N + j]);
                acch[0][e] = addq(acch[0][e], addq(montmul64(xa, ca, q, qinv), montmul64(xb, cpa, q, qinv)));
                acch[1][e] = addq(acch[1][e], addq(montmul64(xa, cb, q, qinv), montmul64(xb, bh, q, qinv)));
            }
            __syncthreads();
        }
        inverse_to_acc(acch);
    }

    if (a.acc_out) {
        int64_t* dst = a.acc_out + (size_t)ct * 2 * N;
        for (int idx = t; idx < 2 * N; idx += H) dst[idx] = (int64_t)acc[idx];
    }
    if (a.big_out) {
        // extractTlweFromTrlwe(out, acc, 0): a'[j] = j ? -a[N-j] : a[0], b' = b[0], rescaled 2^T -> 2^32
        int32_t* dst = a.big_out + (size_t)ct * (N + 1);
        for (int j = t; j <= N; j += H) {
            const TT x = j == N ? acc[N] : (j == 0 ? acc[0] : tneg<T>(acc[N - j]));
            if constexpr (T == 32) dst[j] = (int32_t)x;
            else dst[j] = (int32_t)modswitch_down((int64_t)x, T - 32, 32);
        }
    }
}

// blindRotateNtt (yatfhe/src/blind_rotate.cpp:549-560) on the group-g key family, after
// genNoiselessTrlweSample (or from a given accumulator), and the extraction; one ciphertext
// per CTA of N/2 threads, thread t owning coefficients and slots t and t + N/2, the reference's
// arithmetic mod q as in lazy_blind_rotate_kernel.  Per step the accumulator's digit
// polynomials of the L used levels (digits of its l_full-level decomposition,
// gadgetDecomposeTrlwe) go through one batch of 2L forward transforms, then per slot
//   acc^[o] = sum_(lvl, col) D[lvl][col] . K'[lvl][col][o],
// K' = K_0 + sum_(k2 > 0) NTT(X^(r_k2)) . K_k2 over the group's 2^g keys (rotateTrgswNtt and the
// sums of blindRotateGroup2Ntt / Group3Ntt; r_k2 the sum of the a's whose bit is set in k2),
// NTT(X^r) in slot s being psi^(r e_s) (a table lookup), then one inverse batch of 2.
// Group 1 is the CMux of blindRotateNormalNtt: acc += EP(K_i, X^(a_i) acc - acc) for a_i != 0.
template <int T>
__global__ void __launch_bounds__(1024, 1) group_blind_rotate_kernel(const GroupBrArgs a) {
    using TT = typename TorusOf<T>::type;
    using U = typename TorusOf<T>::utype;
    extern __shared__ __align__(16) unsigned char gr_smem[];
    const int N = a.N, H = N >> 1, t = threadIdx.x, n = a.n, L = a.L, rb = a.radix_bits;
    const int logN = 31 - __clz(N);
    const int ct = blockIdx.x;
    const int g = a.group, G = 1 << g;
    const uint64_t q = a.q, qinv = a.qinv, q2 = 2 * q;
    uint64_t* sw = reinterpret_cast<uint64_t*>(gr_smem);                  // [2L][N]
    TT* acc = reinterpret_cast<TT*>(sw + (size_t)2 * L * N);              // [2][N]
    int16_t* sa = reinterpret_cast<int16_t*>(acc + 2 * N);                // [n + 1]
    const int jj[2] = {t, t + H};
    const size_t keyw = (size_t)L * 4 * N;  // words of one key's used levels

    auto lift = [q](int64_t x) -> uint64_t { return x < 0 ? (uint64_t)(x + (int64_t)q) : (uint64_t)x; };
    auto addq = [q](uint64_t x, uint64_t y) -> uint64_t {
        const uint64_t s = x + y;
        return s >= q ? s - q : s;
    };
    auto red4 = [q, q2](uint64_t x) -> uint64_t {
        x = x >= q2 ? x - q2 : x;
        return x >= q ? x - q : x;
    };
    auto to_torus = [&](uint64_t v) -> TT {
        v = mulshoup64(v, a.post, a.postp, q);
        const int64_t c = v >= (q + 1) / 2 ? (int64_t)(v - q) : (int64_t)v;
        if constexpr (T == 32) return (int32_t)(uint32_t)(uint64_t)c;
        else return sext<56>(c);
    };
    auto norm = [N](int r) {
        r %= 2 * N;
        return r < 0 ? r + 2 * N : r;
    };
    // (X^r p)[j] for r in [0, 2N) (rotateTorusPolynomial, yatfhe/src/polynomial.cpp:184-193)
    auto rot_at = [N](const TT* p, int r, int j) -> TT {
        int x = j - r;
        bool neg = false;
        if (x < 0) {
            x += N;
            neg = true;
        }
        if (x < 0) {
            x += N;
            neg = false;
        }
        const TT v = p[x];
        return neg ? tneg<T>(v) : v;
    };

    // rescaleTlweToNewMod into mod 2N (yatfhe/src/tlwe.cpp:75-81), unless given already scaled
    if (a.scaled_in) {
        const int32_t* in = a.scaled_in + (size_t)ct * n;
        for (int i = t; i < n; i += H) sa[i] = (int16_t)in[i];
    } else {
        const int32_t* in = a.lwe_in + (size_t)ct * (n + 1);
        for (int i = t; i <= n; i += H) sa[i] = (int16_t)modswitch_down(in[i], 31 - logN, logN + 1);
    }
    __syncthreads();
    if (a.acc_in) {
        const int64_t* src = a.acc_in + (size_t)ct * 2 * N;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            acc[jj[e]] = (TT)src[jj[e]];
            acc[N + jj[e]] = (TT)src[N + jj[e]];
        }
    } else {
        // genNoiselessTrlweSample (yatfhe/src/trlwe.cpp:175-182): (0, X^(-b) v)
        const int rb0 = norm(-(int)sa[n]);
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int j = jj[e];
            int x = j - rb0;
            bool neg = false;
            if (x < 0) {
                x += N;
                neg = true;
            }
            if (x < 0) {
                x += N;
                neg = false;
            }
            const TT v = (TT)a.lut[x];
            acc[j] = 0;
            acc[N + j] = neg ? tneg<T>(v) : v;
        }
    }
    __syncthreads();

    const int steps = g == 1 ? n : n / g;
    for (int s = 0; s < steps; ++s) {
        int r1 = 0;
        int rots[8];
        if (g == 1) {
            const int ai = sa[s];
            if (ai == 0) continue;  // the same for every thread of the CTA
            r1 = norm(ai);
        } else {
            for (int k2 = 1; k2 < G; ++k2) {
                int r = 0;
                for (int i2 = 0; i2 < g; ++i2)
                    if ((k2 >> (g - 1 - i2)) & 1) r += sa[s * g + i2];
                rots[k2] = norm(r);
            }
        }
        // the input's digit polynomials of the used levels (group 1: of X^a acc - acc)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int j = jj[e];
#pragma unroll
            for (int poly = 0; poly < 2; ++poly) {
                const TT* p = acc + poly * N;
                const TT x = g == 1 ? tsub<T>(rot_at(p, r1, j), p[j]) : p[j];
                zero_mean_digits<U, T>((U)x, a.l_full, rb, [&](int level, int d) {
                    if (level < L) sw[(size_t)(level * 2 + poly) * N + j] = lift(d);
                });
            }
        }
        __syncthreads();
        q_forward_batch(sw, 2 * L, N, logN, a.wf, a.wfp, q);
        uint64_t h[2][2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int j = jj[e];
            uint64_t R[8];
            if (g > 1) {
                const int ej = (int)a.slot_exp[j];
                for (int k2 = 1; k2 < G; ++k2) R[k2] = a.psi_m[(rots[k2] * ej) & (2 * N - 1)];
            }
            const uint64_t* kb = a.key + (size_t)s * (g == 1 ? 1 : G) * keyw + j;
            uint64_t h0 = 0, h1 = 0;
            // unrolled by 3: the key loads of three levels are in flight together (the loop is
            // bound by L2 latency; +1.4 % for group 2 at 9,728 ciphertexts, bit-identical)
#pragma unroll 3
            for (int lvl = 0; lvl < L; ++lvl)
#pragma unroll
                for (int col = 0; col < 2; ++col) {
                    const uint64_t X = red4(sw[(size_t)(lvl * 2 + col) * N + j]);
                    const size_t off = (size_t)((lvl * 2 + col) * 2) * N;
                    uint64_t k0 = kb[off], k1 = kb[off + N];
                    for (int k2 = 1; k2 < (g == 1 ? 1 : G); ++k2) {
                        k0 = addq(k0, montmul64(R[k2], kb[(size_t)k2 * keyw + off], q, qinv));
                        k1 = addq(k1, montmul64(R[k2], kb[(size_t)k2 * keyw + off + N], q, qinv));
                    }
                    h0 = addq(h0, montmul64(X, k0, q, qinv));
                    h1 = addq(h1, montmul64(X, k1, q, qinv));
                }
            h[0][e] = h0;
            h[1][e] = h1;
        }
        __syncthreads();
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) sw[poly * N + jj[e]] = h[poly][e];
        __syncthreads();
        q_inverse_batch(sw, 2, N, logN, a.wi, a.wip, q);
#pragma unroll
        for (int poly = 0; poly < 2; ++poly)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const TT r = to_torus(sw[poly * N + jj[e]]);
                TT& dst = acc[poly * N + jj[e]];
                dst = g == 1 ? tadd<T>(dst, r) : r;  // accumulateTrlwe for the CMux
            }
        __syncthreads();
    }

    if (a.acc_out) {
        int64_t* dst = a.acc_out + (size_t)ct * 2 * N;
        for (int idx = t; idx < 2 * N; idx += H) dst[idx] = (int64_t)acc[idx];
    }
    if (a.big_out) {
        int32_t* dst = a.big_out + (size_t)ct * (N + 1);
        for (int j = t; j <= N; j += H) {
            const TT x = j == N ? acc[N] : (j == 0 ? acc[0] : tneg<T>(acc[N - j]));
            if constexpr (T == 32) dst[j] = (int32_t)x;
            else dst[j] = (int32_t)modswitch_down((int64_t)x, T - 32, 32);
        }
    }
}

// Teams of one ciphertext slice: one per RNS channel (kLayoutChannel), or one per channel
// and accumulator row (kLayoutChannelRow).
template <int SPLIT>
__host__ __device__ constexpr int slice_teams() { return SPLIT ? 2 * kChannels : kChannels; }
template <int LOGN, int SPLIT>
__host__ __device__ constexpr int slice_threads() { return slice_teams<SPLIT>() * TeamShape<LOGN>::S; }

// Register cap of the blind-rotation kernels: 168 lets four 3-warp slices (or two 6-warp
// ones) share an SM.  (A lower cap for more resident warps measured slower: the kernel
// spills or loses more to its smaller instruction window than the extra warps hide.)
constexpr int kBrMaxRegs = 168;

// Barrier over the two teams of one channel in the channel-row layout: named barrier
// `id` (1..15; 0 is __syncthreads) over their 2 S threads.
template <int LOGN>
__device__ __forceinline__ void pair_sync(int id) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(2 * TeamShape<LOGN>::S) : "memory");
}

// G ciphertexts (slices) per CTA share its L1: slices under one key read the same key lines
// at about the same time, the first from L2 and the others from L1.  Each slice
// synchronises only its own threads, so the slices drift apart freely (measured faster than
// running them in lockstep under CTA-wide barriers).
//
// Layouts (SPLIT):
//   kLayoutChannel     one team per RNS channel runs all 2 l forward NTTs of a CMux step,
//                      the MAC into both output polys and both inverse NTTs;
//   kLayoutChannelRow  two teams per channel, one per accumulator row: each runs the l
//                      forward NTTs of its row's digits and accumulates partial products
//                      for both outputs, the teams swap the partial sum the other one
//                      finishes through shared memory, and each runs one inverse NTT.
//                      Twice the threads per ciphertext, about half the time per step.
template <int LOGN, int T, int G, int SPLIT>
__global__ void __maxnreg__(kBrMaxRegs) blind_rotate_kernel(const BrArgs a) {
    using Sh = TeamShape<LOGN>;
    using TorusT = typename TorusOf<T>::type;
    using U = typename TorusOf<T>::utype;
    constexpr int N = Sh::N, S = Sh::S;
    constexpr int TEAMS = slice_teams<SPLIT>();
    constexpr int PS = prime_set_for(T);  // the context's RNS primes (rns.cuh)
    constexpr int ST = slice_threads<LOGN, SPLIT>();
    extern __shared__ __align__(16) unsigned char smem[];

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int g = warp / (TEAMS * Sh::WARPS);               // ciphertext slice of this warp
    const int wi = warp % (TEAMS * Sh::WARPS);
    const int tm = wi / Sh::WARPS;                           // team in the slice
    const int team = SPLIT ? tm >> 1 : tm;                   // RNS channel
    const int hrow = SPLIT ? tm & 1 : 0;                     // accumulator row (channel-row layout)
    const int tt = (wi % Sh::WARPS) * 32 + lane;             // thread in the team
    const int bar = g * TEAMS + tm;                          // named barrier of the team (N = 2048)
    // named barrier of the channel's team pair, after the team barriers
    const int pair_bar = 1 + (LOGN == 10 ? 0 : G * TEAMS) + g * kChannels + team;
    const int ltid = tid - g * ST;                           // thread in the slice
    // barrier over this slice's threads (the CTA's when it holds one slice): slices of a CTA
    // run independently and only share the L1
    const int slice_bar = 1 + (LOGN == 10 ? 0 : G * TEAMS) + (SPLIT ? G * kChannels : 0) + g;
    auto slice_sync = [&]() {
        if constexpr (G == 1) __syncthreads();
        else asm volatile("bar.sync %0, %1;" ::"r"(slice_bar), "r"(ST) : "memory");
    };
    const Chan ch = pick_chan(a.ch, team);
    const int L = a.L, n = a.n;
    const uint64_t keep = l2_evict_last_policy();

    // the slice's shared memory: xb[team][o] padded regions (NTT transpose scratch, then
    // inverse-NTT residues for the CRT), the accumulator, the digits, the mod-2N input
    unsigned char* base = smem + (size_t)g * br_smem_bytes(LOGN, T, n, L, SPLIT);
    uint32_t* xb = reinterpret_cast<uint32_t*>(base);                           // [3][2][TBUF]
    TorusT* acc = reinterpret_cast<TorusT*>(xb + kChannels * 2 * Sh::TBUF);    // [2][N]
    // digit rows decomposed per phase: both at T = 32 and in the channel-row layout; one at
    // a time at T = 56, where the halved digit buffer lets two ciphertext slices share an SM
    constexpr int DROWS = SPLIT ? 2 : digit_rows(T);
    int16_t* dig = reinterpret_cast<int16_t*>(acc + 2 * N);                     // [DROWS][L][N]
    int16_t* sa = dig + DROWS * L * N;                                           // [n+1]
    // T = 32: the digit-product tables of the forward transforms' first two stages,
    // [3][kTab0Tables][kTab0Words]: w d mod p for w = w1, w2, w1 w2, w3, w1 w3 (ntt.cuh, TAB = 2)
    uint32_t* tab0 = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(sa + n + 1) + 3) & ~(uintptr_t)3);
    const bool use_tab0 = T == 32 && a.radix_bits <= 7;
    static_assert(kTab0Words == kTab0WordsNtt, "one table stride");
    if (use_tab0) {
        constexpr int D = 2 * kTab0Half + 1;
        for (int idx = ltid; idx < kChannels * kTab0Tables * D; idx += ST) {
            const int c = idx / (kTab0Tables * D), t = (idx / D) % kTab0Tables, d = idx % D - kTab0Half;
            const int64_t pc = pick_chan(a.ch, c).p;
            const int64_t w1 = c_tw_head[PS][LOGN - 10][c][0][1].x, w2 = c_tw_head[PS][LOGN - 10][c][0][2].x;
            const int64_t w3 = c_tw_head[PS][LOGN - 10][c][0][3].x;
            const int64_t w = t == 0 ? w1 : t == 1 ? w2 : t == 2 ? w1 * w2 % pc : t == 3 ? w3 : w1 * w3 % pc;
            const int64_t v = w * d % pc;
            tab0[(c * kTab0Tables + t) * kTab0Words + kTab0Half + d] = (uint32_t)(v < 0 ? v + pc : v);
        }
    }
    // the team's transpose region: region 0 of its channel (channel layout, the inverse
    // uses both), or region `hrow` (channel-row layout, each team owns one)
    uint32_t* mine = xb + (team * 2 + hrow) * Sh::TBUF;

    // one digit polynomial of this team's channel into x, forward transform
    auto load_and_forward = [&](uint32_t (&x)[32], const int16_t* d) {
        if constexpr (T == 32) {
            if (use_tab0) {
#pragma unroll
                for (int r = 0; r < 32; ++r) x[r] = (uint32_t)(int32_t)d[r * S + tt];
                ntt_forward<LOGN, PS, 2>(x, mine, tt, team, bar, ch, tab0 + team * kTab0Tables * kTab0Words + kTab0Half);
                return;
            }
        }
        const uint32_t bias = fwd_bias_digits<LOGN, PS>(ch.p);
#pragma unroll
        for (int r = 0; r < 32; ++r) x[r] = (uint32_t)(int32_t)d[r * S + tt] + bias;
        ntt_forward<LOGN, PS>(x, mine, tt, team, bar, ch);
    };

    // G ciphertexts per iteration; a grid smaller than the batch makes the CTAs persistent
    for (int first = blockIdx.x * G; first < a.count; first += gridDim.x * G) {
    const int ct = first + g;
    const bool valid = ct < a.count;
    const uint4* key = !valid ? nullptr : (a.key_of ? a.key_table[a.key_of[ct]] : a.key);
    const int64_t* lut = !valid ? nullptr : (a.lut_of ? a.lut_table[a.lut_of[ct]] : a.lut);

    // rescaleTlweToNewMod into mod 2N (yatfhe/src/tlwe.cpp:75-81), unless given already scaled
    if (valid) {
        if (a.scaled_in) {
            const int32_t* in = a.scaled_in + (size_t)ct * n;
            for (int i = ltid; i < n; i += ST) sa[i] = (int16_t)in[i];
        } else {
            const int32_t* in = a.lwe_in + (size_t)ct * (n + 1);
            for (int i = ltid; i <= n; i += ST) sa[i] = (int16_t)modswitch_down(in[i], 31 - LOGN, LOGN + 1);
        }
    }
    slice_sync();

    if (valid) {
        if (a.acc_in) {
            const int64_t* src = a.acc_in + (size_t)ct * 2 * N;
            for (int idx = ltid; idx < 2 * N; idx += ST) acc[idx] = (TorusT)src[idx];
        } else {
            // genNoiselessTrlweSample: acc = (0, X^-b v) (yatfhe/src/trlwe.cpp:175-182)
            int t2 = -(int)sa[n];
            t2 = ((t2 % (2 * N)) + 2 * N) % (2 * N);
            const bool wrap = t2 >= N;
            const int at = wrap ? t2 - N : t2;
            for (int j = ltid; j < N; j += ST) {
                acc[j] = 0;
                TorusT v = j < at ? tneg<T>((TorusT)lut[j - at + N]) : (TorusT)lut[j - at];
                acc[N + j] = wrap ? tneg<T>(v) : v;
            }
        }
    }
    slice_sync();

    for (int i = 0; i < a.steps; ++i) {
        const int ai = valid ? (int)sa[i] : 0;
        // a_i == 0 leaves the accumulator unchanged (the skip of blind_rotate.cpp:1557); with
        // one ciphertext per CTA the whole step is skipped, otherwise only its work
        if (G == 1 && ai == 0) continue;
        const bool active = ai != 0;
        const int t2 = ai < 0 ? ai + 2 * N : ai;
        const bool wrap = t2 >= N;
        const int at = wrap ? t2 - N : t2;
        // externalProductTrgswMPNttImpl (yatfhe/src/trgsw.cpp:712-767) in channel `team`:
        // forward NTT of every digit poly, Montgomery MAC against the key, inverse NTT.
        uint32_t oa[32], ob[32];
        const uint32_t pinv = 0u - ch.pinv_neg;
#pragma unroll
        for (int r = 0; r < 32; ++r) oa[r] = ob[r] = 0;
#pragma unroll 1
        for (int row0 = 0; row0 < 2; row0 += DROWS) {
            // tmp = X^{a_i} acc - acc (rotateTrlweMinusOne, yatfhe/src/trlwe.cpp:284-289) for
            // DROWS rows, then gadgetDecomposeTrlwe (yatfhe/src/trlwe.cpp:185-198) into int16 digits
            if (active) {
                // LC, RC > 0 fix the level count and radix at compile time (the digit loop
                // unrolls with constant shifts); 0 reads them from the arguments
                auto decompose = [&](auto lc, auto rc) {
                    constexpr int LC = decltype(lc)::value, RC = decltype(rc)::value;
                    const int levels = LC ? LC : L, radix = RC ? RC : a.radix_bits;
                    // two coefficients per iteration: +1.6 % at T = 32 (unroll 4: no gain), the
                    // same at T = 56 (A/B on GB300, outputs identical)
#pragma unroll 2
                    for (int idx = ltid; idx < DROWS * N; idx += ST) {
                        const int dr = idx >= N;
                        const int j = idx - dr * N;
                        const TorusT* A = acc + (row0 + dr) * N;
                        TorusT rot = j < at ? tneg<T>(A[j - at + N]) : A[j - at];
                        if (wrap) rot = tneg<T>(rot);
                        const TorusT tmp = tsub<T>(rot, A[j]);
                        int16_t* d = dig + dr * levels * N + j;
                        zero_mean_digits<U, T>((U)tmp, levels, radix, [&](int level, int v) { d[level * N] = (int16_t)v; });
                    }
                };
                using std::integral_constant;
                if (T == 32 && L == 3 && a.radix_bits == 7)
                    decompose(integral_constant<int, 3>{}, integral_constant<int, 7>{});
                else if (T == 56 && L == 4 && a.radix_bits == 10)
                    decompose(integral_constant<int, 4>{}, integral_constant<int, 10>{});
                else
                    decompose(integral_constant<int, 0>{}, integral_constant<int, 0>{});
            }
            slice_sync();

            if (SPLIT) break;  // the channel-row layout continues below
            if (active) {
                for (int dr = 0; dr < DROWS; ++dr) {
                    const int row = row0 + dr;
                    for (int lvl = 0; lvl < L; ++lvl) {
                        uint32_t x[32];
                        const int16_t* d = dig + ((size_t)dr * L + lvl) * N;
                        load_and_forward(x, d);
                        const uint4* kp =
                            key + ((((size_t)i * L + lvl) * 2 + row) * kChannels + team) * (key_block_words(N) / 4);
#pragma unroll
                        for (int rr = 0; rr < 8; ++rr) {
                            const uint4 ka = ldg_keep(kp + rr * S + tt, keep);
                            const uint4 kb = ldg_keep(kp + (8 + rr) * S + tt, keep);
                            const uint32_t kav[4] = {ka.x, ka.y, ka.z, ka.w};
                            const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w};
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const int r = rr * 4 + e;
                                oa[r] += montdiff<T == 32>(x[r], kav[e], ch.p, pinv);
                                ob[r] += montdiff<T == 32>(x[r], kbv[e], ch.p, pinv);
                            }
                        }
                        // lazy accumulation: each montdiff term lies in (-p, p), so after a
                        // reduction oa, ob in [0, 4p) take two terms ((-2p, 6p)) before the next
                        // one brings (oa + 2p) in (0, 8p) back to [0, 4p); 2 l terms in all (even)
                        if ((row * L + lvl) & 1) {
#pragma unroll
                            for (int r = 0; r < 32; ++r) {
                                oa[r] = reduce_once(oa[r] + ch.two_p, 2 * ch.two_p);
                                ob[r] = reduce_once(ob[r] + ch.two_p, 2 * ch.two_p);
                            }
                        }
                    }
                }
            }
            if (DROWS == 1 && row0 == 0) slice_sync();  // the next row's digits overwrite these
        }
        if constexpr (SPLIT && T == 32) {
            if (active) {
                // this team's row: l forward NTTs.  After each one the two teams of the
                // channel swap their transforms through their own regions, and each
                // accumulates only the output it finishes (row 0 -> a, row 1 -> b) from both
                // rows' digits: per level the two products (< 46p * p each) are summed exactly in
                // 64 bits and reduced once (Montgomery, a term in (-p, 2.1p)); the 32-bit sum
                // starts at l p, so it stays in (0, 3.1 l p), below 2^32 for l <= 15.
                const int row = hrow;
                const uint32_t* other = xb + (team * 2 + (1 - hrow)) * Sh::TBUF;
                uint32_t acc32[32];
#pragma unroll
                for (int r = 0; r < 32; ++r) acc32[r] = L * ch.p;
                for (int lvl = 0; lvl < L; ++lvl) {
                    uint32_t x[32];
                    load_and_forward(x, dig + ((size_t)row * L + lvl) * N);
                    team_sync<LOGN>(bar);  // the team's transpose reads of its region are done
#pragma unroll
                    for (int r = 0; r < 32; ++r) mine[r * S + tt] = x[r];
                    pair_sync<LOGN>(pair_bar);  // the partner's transform is in its region
                    const size_t blk = (size_t)i * L + lvl;
                    const uint4* kown = key + ((blk * 2 + row) * kChannels + team) * (key_block_words(N) / 4) +
                                        (row ? 8 : 0) * S;
                    const uint4* kpar = key + ((blk * 2 + (1 - row)) * kChannels + team) * (key_block_words(N) / 4) +
                                        (row ? 8 : 0) * S;
#pragma unroll
                    for (int rr = 0; rr < 8; ++rr) {
                        const uint4 ka = ldg_keep(kown + rr * S + tt, keep);
                        const uint4 kb = ldg_keep(kpar + rr * S + tt, keep);
                        const uint32_t kav[4] = {ka.x, ka.y, ka.z, ka.w};
                        const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w};
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int r = rr * 4 + e;
                            const uint64_t sp = (uint64_t)x[r] * kav[e] + (uint64_t)other[r * S + tt] * kbv[e];
                            acc32[r] += (uint32_t)(sp >> 32) - __umulhi((uint32_t)sp * pinv, ch.p);
                        }
                    }
                    pair_sync<LOGN>(pair_bar);  // the partner has read this region
                }
                // one Shoup reduction by 1 to [0, 2p) for the inverse transform
                const uint32_t one_s = 0xFFFFFFFFu / ch.p;
#pragma unroll
                for (int r = 0; r < 32; ++r) {
                    const uint32_t t = acc32[r];
                    oa[r] = t - __umulhi(t, one_s) * ch.p;
                }
                ntt_inverse<LOGN, PS>(oa, mine, tt, team, bar, ch);
                team_sync<LOGN>(bar);
#pragma unroll
                for (int r = 0; r < 32; ++r) mine[r * S + tt] = reduce_once(oa[r], ch.p);
            }
        } else if constexpr (SPLIT) {
            if (active) {
                // this team's row: l forward NTTs; oa gathers the output this team finishes
                // (row 0 -> a, row 1 -> b), ob the other output's partial sum
                const int row = hrow;
                for (int lvl = 0; lvl < L; ++lvl) {
                    uint32_t x[32];
                    const int16_t* d = dig + ((size_t)row * L + lvl) * N;
                    load_and_forward(x, d);
                    const uint4* kp =
                        key + ((((size_t)i * L + lvl) * 2 + row) * kChannels + team) * (key_block_words(N) / 4);
                    const uint4* kown = kp + (row ? 8 : 0) * S;
                    const uint4* kother = kp + (row ? 0 : 8) * S;
#pragma unroll
                    for (int rr = 0; rr < 8; ++rr) {
                        const uint4 ka = ldg_keep(kown + rr * S + tt, keep);
                        const uint4 kb = ldg_keep(kother + rr * S + tt, keep);
                        const uint32_t kav[4] = {ka.x, ka.y, ka.z, ka.w};
                        const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w};
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int r = rr * 4 + e;
                            oa[r] += montdiff<T == 32>(x[r], kav[e], ch.p, pinv);
                            ob[r] += montdiff<T == 32>(x[r], kbv[e], ch.p, pinv);
                        }
                    }
                    // lazy accumulation as in the channel layout, reduced after odd levels
                    // and once more at the end when l is odd: [0, 4p) on exit
                    if ((lvl & 1) || lvl == L - 1) {
#pragma unroll
                        for (int r = 0; r < 32; ++r) {
                            oa[r] = reduce_once(oa[r] + ch.two_p, 2 * ch.two_p);
                            ob[r] = reduce_once(ob[r] + ch.two_p, 2 * ch.two_p);
                        }
                    }
                }
                // swap partial sums with the channel's other team: write the one it
                // finishes into this team's region once its transposes are done, wait,
                // add the partner's, wait until the partner has read this region
                team_sync<LOGN>(bar);
#pragma unroll
                for (int r = 0; r < 32; ++r) mine[r * S + tt] = ob[r];
                pair_sync<LOGN>(pair_bar);
                const uint32_t* other = xb + (team * 2 + (1 - hrow)) * Sh::TBUF;
#pragma unroll
                for (int r = 0; r < 32; ++r) oa[r] = reduce_once(reduce_once(oa[r] + other[r * S + tt], 2 * ch.two_p), ch.two_p);
                pair_sync<LOGN>(pair_bar);
                ntt_inverse<LOGN, PS>(oa, mine, tt, team, bar, ch);
                team_sync<LOGN>(bar);
#pragma unroll
                for (int r = 0; r < 32; ++r) mine[r * S + tt] = reduce_once(oa[r], ch.p);
            }
        } else if (active) {
            // one copy of the inverse transform, applied to the a then the b output poly
#pragma unroll 1
            for (int o = 0; o < 2; ++o) {
                if (o == 1) {
#pragma unroll
                    for (int r = 0; r < 32; ++r) oa[r] = ob[r];
                }
                uint32_t* region = mine + o * Sh::TBUF;
#pragma unroll
                for (int r = 0; r < 32; ++r) oa[r] = reduce_once(oa[r], ch.two_p);  // [0, 2p) in
                ntt_inverse<LOGN, PS>(oa, region, tt, team, bar, ch);
                team_sync<LOGN>(bar);
#pragma unroll
                for (int r = 0; r < 32; ++r) region[r * S + tt] = reduce_once(oa[r], ch.p);
            }
        }
        slice_sync();

        // CRT -> applyIntt's centred mod-q value mod 2^T, then accumulateTrlwe (trlwe.h:268-274)
        if (active) {
#pragma unroll 1
            for (int idx = ltid; idx < 2 * N; idx += ST) {
                const int o = idx >= N;
                const int j = idx - o * N;
                const int64_t v = crt_to_torus<T>(xb[(0 * 2 + o) * Sh::TBUF + j], xb[(1 * 2 + o) * Sh::TBUF + j],
                                                  xb[(2 * 2 + o) * Sh::TBUF + j], a.crt);
                if constexpr (T == 32) acc[idx] = (int32_t)((uint32_t)acc[idx] + (uint32_t)v);
                else acc[idx] = sext<56>((int64_t)((uint64_t)acc[idx] + (uint64_t)v));
            }
        }
        slice_sync();
    }

    if (valid && a.acc_out) {
        int64_t* dst = a.acc_out + (size_t)ct * 2 * N;
        for (int idx = ltid; idx < 2 * N; idx += ST) dst[idx] = (int64_t)acc[idx];
    }
    if (valid && a.big_out) {
        // extractTlweFromTrlwe(out, acc, 0): a'[j] = j ? -a[N-j] : a[0], b' = b[0], rescaled 2^T -> 2^32
        int32_t* dst = a.big_out + (size_t)ct * (N + 1);
        for (int j = ltid; j <= N; j += ST) {
            TorusT x = j == N ? acc[N] : (j == 0 ? acc[0] : tneg<T>(acc[N - j]));
            if constexpr (T == 32) dst[j] = (int32_t)x;
            else dst[j] = (int32_t)modswitch_down((int64_t)x, T - 32, 32);
        }
    }
    slice_sync();  // the next ciphertexts reuse the shared-memory state
    }
}

// Row-cluster layout (kLayoutRowCluster), T = 32, N = 1024: one ciphertext per cluster of
// two CTAs.  CTA h (its rank in the cluster) owns accumulator row h (0: a, 1: b) and computes
// output h of every external product; warp w = c L + lvl is the team of RNS channel c and
// digit level lvl.  Per CMux step: (1) all threads rotate and decompose row h into l digit
// rows; (2) each team runs the forward transform of its level's digits and writes it into
// the partner CTA's exchange region of the same team (distributed shared memory; two
// regions used alternately by the active steps, so a region is rewritten only after the
// partner has passed the next cluster barrier); after the cluster barrier (3) each team
// multiplies its transform and the partner's with the key words for output h, an exact
// 64-bit sum of two products reduced once, into its partial region; (4) the level-0 team of
// each channel adds the l partials and runs the inverse transform; (5) all threads
// recombine the channels (CRT) and add into row h.  The levels' transforms run side by
// side, so a step takes about one forward and one inverse transform instead of l forward
// ones: the latency shape for lone ciphertexts.  With l <= kClusterStageLevels the key rows
// a step multiplies with (output h of both rows, every level and channel: 18 x 4 KB at
// l = 3) are copied into shared memory by TMA (cp.async.bulk, one thread, an mbarrier)
// while the previous step's inverse transform, CRT and the step's digits and forward
// transforms run; the wait for them is bounded in time, and a copy that does not arrive
// counts in g_wait_timeouts and the CTA reads the key from global memory from then on.
template <int T>
__global__ void __cluster_dims__(2, 1, 1) __maxnreg__(kBrMaxRegs) blind_rotate_cluster_kernel(const BrArgs a) {
    static_assert(T == 32, "the row-cluster layout is built for the 32-bit torus");
    namespace cg = cooperative_groups;
    using Sh = TeamShape<10>;
    constexpr int N = Sh::N, S = Sh::S;
    constexpr int PS = prime_set_for(T);
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cluster = cg::this_cluster();
    const int h = (int)cluster.block_rank();
    const int L = a.L, n = a.n;
    const int ct = (int)(blockIdx.x >> 1);
    const bool valid = ct < a.count;  // the grid is two CTAs per ciphertext: uniform per cluster
    const int tid = threadIdx.x, NT = blockDim.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int c = warp / L, lvl = warp - c * L;
    const Chan ch = pick_chan(a.ch, c);
    const uint64_t keep = l2_evict_last_policy();
    const uint32_t pinv = 0u - ch.pinv_neg;
    const uint32_t one_s = 0xFFFFFFFFu / ch.p;  // floor(2^32 / p): Shoup reduction by 1

    const size_t team_words = (size_t)kChannels * L * Sh::TBUF;
    // [3][L][TBUF]: transposes, then the partial sums (step 3), then the inverse outputs
    uint32_t* regions = reinterpret_cast<uint32_t*>(smem);
    uint32_t* exch = regions + team_words;                  // [2][3][L][TBUF] written by the partner
    int32_t* acc = reinterpret_cast<int32_t*>(exch + 2 * team_words);  // [N] row h
    int16_t* dig = reinterpret_cast<int16_t*>(acc + N);               // [L][N]
    int16_t* sa = dig + (size_t)L * N;                                // [n+1]
    uint32_t* tab0 = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(sa + n + 1) + 3) & ~(uintptr_t)3);
    uint32_t* mine = regions + (size_t)(c * L + lvl) * Sh::TBUF;
    uint32_t* part = mine;  // the team's transpose region holds its partial sum after step 3
    uint32_t* stage = reinterpret_cast<uint32_t*>(smem + brc_stage_offset(n, L));  // [L][2][3][1024]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + brc_smem_bytes(n, L) - 16);
    volatile int* stage_ok = reinterpret_cast<volatile int*>(mbar + 1);
    const uint32_t mbar_a = (uint32_t)__cvta_generic_to_shared(mbar);
    uint32_t* my_exch = exch + (size_t)(c * L + lvl) * Sh::TBUF;     // + ph * team_words
    uint32_t* their_exch = cluster.map_shared_rank(my_exch, 1 - h);  // the partner CTA's same team
    int ph = 0;                                                      // exchange region of this step

    const uint4* key = !valid ? nullptr : (a.key_of ? a.key_table[a.key_of[ct]] : a.key);
    const int64_t* lut = !valid ? nullptr : (a.lut_of ? a.lut_table[a.lut_of[ct]] : a.lut);
    // TMA stage of the key rows (uniform in the cluster; nothing runs for an invalid one)
    bool tma = valid && L <= kClusterStageLevels;
    if (tma && tid == 0) {
        mbar_init(mbar_a, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // thread 0: arms the barrier and copies key rows of `step` (output h) into the stage
    auto issue = [&](int step) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(mbar_a, (uint32_t)L * 2 * kChannels * 4096);
        for (int lv = 0; lv < L; ++lv)
            for (int row = 0; row < 2; ++row)
                for (int cc = 0; cc < kChannels; ++cc) {
                    const size_t blk = (size_t)step * L + lv;
                    const uint4* src =
                        key + ((blk * 2 + row) * kChannels + cc) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
                    bulk_copy_g2s((uint32_t)__cvta_generic_to_shared(stage + ((lv * 2 + row) * kChannels + cc) * 1024),
                                  src, 4096, mbar_a);
                }
    };
    auto next_active = [&](int from) {
        while (from < a.steps && sa[from] == 0) ++from;
        return from;
    };
    uint32_t phase = 0;          // parity of the stage's next barrier phase
    bool outstanding = false;    // thread 0: a copy issued and not yet waited for
    const bool use_tab0 = a.radix_bits <= 7;
    if (use_tab0) {
        for (int idx = tid; idx < kChannels * 129; idx += NT) {
            const int cc = idx / 129, d = idx - cc * 129 - 64;
            const uint32_t pc = pick_chan(a.ch, cc).p;
            const int64_t v = (int64_t)c_tw_head[PS][0][cc][0][1].x * d % pc;
            tab0[cc * 132 + 64 + d] = (uint32_t)(v < 0 ? v + pc : v);
        }
    }
    if (valid) {
        if (a.scaled_in) {
            for (int i = tid; i < n; i += NT) sa[i] = (int16_t)a.scaled_in[(size_t)ct * n + i];
        } else {
            const int32_t* in = a.lwe_in + (size_t)ct * (n + 1);
            for (int i = tid; i <= n; i += NT) sa[i] = (int16_t)modswitch_down(in[i], 31 - 10, 11);
        }
    } else {
        for (int i = tid; i <= n; i += NT) sa[i] = 0;
    }
    __syncthreads();
    if (tma && tid == 0) {
        const int f = next_active(0);
        if (f < a.steps) {
            issue(f);
            outstanding = true;
        }
    }
    if (valid && a.acc_in) {
        for (int j = tid; j < N; j += NT) acc[j] = (int32_t)a.acc_in[(size_t)ct * 2 * N + h * N + j];
    } else if (valid) {
        // genNoiselessTrlweSample: acc = (0, X^-b v) (yatfhe/src/trlwe.cpp:175-182)
        int t2 = -(int)sa[n];
        t2 = ((t2 % (2 * N)) + 2 * N) % (2 * N);
        const bool wrap = t2 >= N;
        const int at = wrap ? t2 - N : t2;
        for (int j = tid; j < N; j += NT) {
            int32_t v = j < at ? tneg<T>((int32_t)lut[j - at + N]) : (int32_t)lut[j - at];
            acc[j] = h == 0 ? 0 : (wrap ? tneg<T>(v) : v);
        }
    } else {
        for (int j = tid; j < N; j += NT) acc[j] = 0;
    }
    cluster.sync();  // the partner has started: its shared memory may be written from here on

    for (int i = 0; i < a.steps; ++i) {
        const int ai = (int)sa[i];
        if (ai == 0) continue;  // the a_i = 0 skip (blind_rotate.cpp:1557), the same in both CTAs
        const int t2 = ai < 0 ? ai + 2 * N : ai;
        const bool wrap = t2 >= N;
        const int at = wrap ? t2 - N : t2;
        // without the stage: this step's key lines of the team (step 3 reads them), requested
        // now so that they arrive in L1 while the digits and the forward transform are computed
        if (!tma) {
            const size_t blk = (size_t)i * L + lvl;
            const uint4* po = key + ((blk * 2 + h) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S + lane;
            const uint4* pp = key + ((blk * 2 + (1 - h)) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S + lane;
#pragma unroll
            for (int rr = 0; rr < 8; ++rr) {
                asm volatile("prefetch.global.L1 [%0];" ::"l"(po + rr * S));
                asm volatile("prefetch.global.L1 [%0];" ::"l"(pp + rr * S));
            }
        }
        // (1) X^{a_i} row - row, zero-mean digits (rotateTrlweMinusOne, gadgetDecomposeTrlwe)
        auto decompose = [&](auto lc, auto rc) {
            constexpr int LC = decltype(lc)::value, RC = decltype(rc)::value;
            const int levels = LC ? LC : L, radix = RC ? RC : a.radix_bits;
#pragma unroll 1
            for (int j = tid; j < N; j += NT) {
                int32_t rot = j < at ? tneg<T>(acc[j - at + N]) : acc[j - at];
                if (wrap) rot = tneg<T>(rot);
                const int32_t tmp = tsub<T>(rot, acc[j]);
                int16_t* d = dig + j;
                zero_mean_digits<uint32_t, 32>((uint32_t)tmp, levels, radix, [&](int level, int v) { d[level * N] = (int16_t)v; });
            }
        };
        if (L == 3 && a.radix_bits == 7)
            decompose(std::integral_constant<int, 3>{}, std::integral_constant<int, 7>{});
        else
            decompose(std::integral_constant<int, 0>{}, std::integral_constant<int, 0>{});
        __syncthreads();
        // (2) this team's forward transform, written into the partner's exchange region
        uint32_t x[32];
        const int16_t* d = dig + (size_t)lvl * N;
        if (use_tab0) {
#pragma unroll
            for (int r = 0; r < 32; ++r) x[r] = (uint32_t)(int32_t)d[r * S + lane];
            ntt_forward<10, PS, 1>(x, mine, lane, c, 0, ch, tab0 + c * 132 + 64);
        } else {
            const uint32_t bias = fwd_bias_digits<10, PS>(ch.p);
#pragma unroll
            for (int r = 0; r < 32; ++r) x[r] = (uint32_t)(int32_t)d[r * S + lane] + bias;
            ntt_forward<10, PS>(x, mine, lane, c, 0, ch);
        }
        {
            uint32_t* dst = their_exch + (size_t)ph * team_words;
#pragma unroll
            for (int r = 0; r < 32; ++r) dst[r * S + lane] = x[r];
        }
        // (3) output h: own row with K(lvl, h, h), the partner's row with K(lvl, 1-h, h);
        // x < 46p and key words < p: the sum of two products fits 64 bits.  The own row's
        // products are formed while the partner may still be transforming.
        const size_t blk = (size_t)i * L + lvl;
        const uint4* gown = key + ((blk * 2 + h) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
        const uint4* gpar = key + ((blk * 2 + (1 - h)) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
        uint64_t own[32];
        // with the stage every thread waits for the step's copies (bounded); a thread that
        // gives up reads the same key words from global memory
        bool from_stage = false;
        if (tma) {
            from_stage = mbar_wait_bounded(mbar_a, phase, kWaitCycles);
            if (!from_stage) atomicAdd(&g_wait_timeouts, 1ull);
            if (tid == 0) {
                if (from_stage) outstanding = false;
                *stage_ok = from_stage;
            }
        }
        const uint4* kown = from_stage ? reinterpret_cast<const uint4*>(stage + ((lvl * 2 + h) * kChannels + c) * 1024) : nullptr;
        const uint4* spar = from_stage ? reinterpret_cast<const uint4*>(stage + ((lvl * 2 + (1 - h)) * kChannels + c) * 1024) : nullptr;
#pragma unroll
        for (int rr = 0; rr < 8; ++rr) {
            const uint4 ka = from_stage ? kown[rr * S + lane] : ldg_keep(gown + rr * S + lane, keep);
            const uint32_t kav[4] = {ka.x, ka.y, ka.z, ka.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) own[rr * 4 + e] = (uint64_t)x[rr * 4 + e] * kav[e];
        }
        cluster.sync();  // both CTAs' transforms are in the partner's exchange regions
        const uint32_t* theirs = my_exch + (size_t)ph * team_words;
        ph ^= 1;
#pragma unroll
        for (int rr = 0; rr < 8; ++rr) {
            const uint4 kb = from_stage ? spar[rr * S + lane] : ldg_keep(gpar + rr * S + lane, keep);
            const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int r = rr * 4 + e;
                const uint64_t s = own[r] + (uint64_t)theirs[r * S + lane] * kbv[e];
                // s 2^-32 mod p (Montgomery) + p: in (0, 3.1p), reduced after the level sum
                part[r * S + lane] = (uint32_t)(s >> 32) - __umulhi((uint32_t)s * pinv, ch.p) + ch.p;
            }
        }
        __syncthreads();  // every partial is written, and the stage has been read
        if (tma) {
            // the copy for the next active step runs while this step finishes
            tma = *stage_ok;  // after thread 0 gave up the CTA reads the key from global memory
            phase ^= 1;
            if (tma && tid == 0) {
                const int f = next_active(i + 1);
                if (f < a.steps) {
                    issue(f);
                    outstanding = true;
                }
            }
        }
        // (4) the level-0 team of each channel: sum of the l partials, inverse transform
        if (lvl == 0) {
            uint32_t oa[32];
#pragma unroll
            for (int r = 0; r < 32; ++r) {
                uint32_t v = 0;
                // unrolled to the largest level count, so the loads issue together
#pragma unroll
                for (int q = 0; q < kClusterMaxLevels; ++q)
                    if (q < L) v += regions[(size_t)(c * L + q) * Sh::TBUF + r * S + lane];
                oa[r] = v - __umulhi(v, one_s) * ch.p;  // l terms < 3.1p each: < 13p; reduced to [0, 2p)
            }
            ntt_inverse<10, PS>(oa, mine, lane, c, 0, ch);
            __syncwarp();
#pragma unroll
            for (int r = 0; r < 32; ++r) mine[r * S + lane] = reduce_once(oa[r], ch.p);
        }
        __syncthreads();
        // (5) CRT -> applyIntt's centred mod-q value mod 2^32, accumulateTrlwe on row h
#pragma unroll 1
        for (int j = tid; j < N; j += NT) {
            const int64_t v = crt_to_torus<T>(regions[(size_t)(0 * L) * Sh::TBUF + j], regions[(size_t)(1 * L) * Sh::TBUF + j],
                                              regions[(size_t)(2 * L) * Sh::TBUF + j], a.crt);
            acc[j] = (int32_t)((uint32_t)acc[j] + (uint32_t)v);
        }
        __syncthreads();
    }

    if (valid && a.acc_out) {
        int64_t* dst = a.acc_out + (size_t)ct * 2 * N + h * N;
        for (int j = tid; j < N; j += NT) dst[j] = (int64_t)acc[j];
    }
    if (valid && a.big_out) {
        // extractTlweFromTrlwe(out, acc, 0): a'[j] = j ? -a[N-j] : a[0] from row 0, b' = b[0] from row 1
        int32_t* dst = a.big_out + (size_t)ct * (N + 1);
        if (h == 0) {
            for (int j = tid; j < N; j += NT) dst[j] = j == 0 ? acc[0] : tneg<T>(acc[N - j]);
        } else if (tid == 0) {
            dst[N] = acc[0];
        }
    }
    // a copy that timed out may still land: wait for it (bounded) before the CTA exits
    if (outstanding && tid == 0 && !mbar_wait_bounded(mbar_a, phase ^ 1, kWaitCycles)) atomicAdd(&g_wait_timeouts, 1ull);
    cluster.sync();  // neither CTA leaves while the other may still write into its regions
}

// Point-to-point signalling between the CTAs of a cluster: a bulk copy (TMA) from this CTA's
// shared memory into another CTA's that completes its bytes on an mbarrier there, so the
// receiver waits for exactly the data it needs instead of a cluster-wide barrier.
__device__ __forceinline__ uint32_t cluster_addr(uint32_t local, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}
// `bytes` (a multiple of 16) from this CTA's shared memory at `src` to the cluster address
// `dst`, completing them on the mbarrier at the cluster address `bar` (16-byte aligned both)
__device__ __forceinline__ void bulk_s2c(uint32_t dst, uint32_t src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "r"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// Waits (at most `cycles` clocks) for a phase completed by other CTAs' copies.
__device__ __forceinline__ bool mbar_wait_cluster_bounded(uint32_t bar, uint32_t parity, long long cycles) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, "
            "0, p;\n}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > cycles) return false;
    }
}
// Word offset of lane l's 16-byte chunk k (its slots 4k..4k+3) in a [32 lanes][32 words]
// region: the eight lanes of a quarter warp reach eight different bank quads.
__device__ __forceinline__ int swz(int l, int k) { return l * 32 + 4 * (k ^ (l & 7)); }
// The same for the 64 threads of a two-warp team with four chunks each ([64][16 words]).
__device__ __forceinline__ int swz16(int tt, int k) { return tt * 16 + 4 * (k ^ ((tt >> 1) & 3)); }

// Channel-cluster layout (kLayoutChannelCluster), T = 32, N = 1024: one ciphertext per
// cluster of six CTAs of eight warps.  CTA (h, c), rank 3 h + c, owns accumulator row h in RNS
// channel c and computes output h of every external product in that channel.  Per CMux
// step: (1) all threads rotate and decompose row h into l digit rows (the three CTAs of a
// row compute the same digits); (2) warp lvl < l runs the forward transform of digit level
// lvl, writes it into its send buffer and one lane copies that (cp.async.bulk, shared memory
// to shared memory) into the exchange region of the same level in the partner CTA (the other
// row, the same channel), completing the partner's barrier for that level; (3) warp lvl and
// its helper warp 4 + lvl (which reads slots 16..31 of each lane from the send buffer) each
// multiply their half of the transform with the key words K(lvl, h, h) and, once the
// partner's transform is in, the partner's half with K(lvl, 1 - h, h): an exact 64-bit sum
// of two products reduced once, added into the levels' partial sum with shared-memory atomic
// adds; (4) warps 0 and 1 run the inverse transform on the partial sum, write row h's
// residues in channel c into the CTA's inbox and copy them into the inboxes of the two other
// CTAs of row h; (5) once the two other channels' residues are in, every thread recombines
// four coefficients (CRT) and adds them into the CTA's copy of row h.  No scheduler runs more
// than one transform warp (the row-cluster layout puts nine on an SM's four), so a step costs
// about one forward and one inverse transform of a warp running alone, and no step waits at a
// cluster-wide barrier.  The inverse runs with 16 residues per thread (ntt16_inverse: half
// the per-thread chain, on schedulers no other warp uses then); warps 0 and 1 read the summed
// partials in its slot order (slot16) and write their residues in 16-byte chunks (thread tt's
// chunk k holds its coefficients (4k + e) 64 + tt, swz16), and thread (tt, k) of the
// recombination takes those.  Two-warp forward transforms measured slower: six transform
// warps on four schedulers put two on two of them.  Send buffers, exchange regions and
// inboxes are double-buffered by the parity of the active step: another CTA's copy for step
// u + 2 depends, through the chain of transforms and recombinations, on this CTA having
// finished step u, so a buffer is rewritten only after it was read (and a send buffer only
// after its copy arrived).  The key rows of the next active step (output h of both rows,
// every level, channel c: l x 2 x 4 KB) are copied into shared memory by TMA from lane 0 of
// warp 7, which runs no transform: it issues the copy once the step's products have read the
// stage, waits for it (bounded) while the inverse runs, and publishes whether it arrived; the
// products read the key from global memory after a wait gave up.  Every wait is bounded; a
// wait for another CTA that gives up counts in g_wait_timeouts (the results are then wrong)
// and the CTA stops waiting.
template <int T>
__global__ void __cluster_dims__(6, 1, 1) __maxnreg__(kBrMaxRegs) blind_rotate_cluster6_kernel(const BrArgs a) {
    static_assert(T == 32, "the channel-cluster layout is built for the 32-bit torus");
    namespace cg = cooperative_groups;
    using Sh = TeamShape<10>;
    constexpr int N = Sh::N, S = Sh::S;
    constexpr int PS = prime_set_for(T);
    constexpr int NT = kCluster6Warps * 32;  // the recombination gives each thread one 16-byte chunk
    static_assert(kCluster6Warps == 8, "eight warps: one per chunk column of the swizzled regions");
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int h = rank / 3, c = rank - 3 * h;
    const int L = a.L, n = a.n;
    const int ct = (int)(blockIdx.x / 6);
    const bool valid = ct < a.count;  // the grid is six CTAs per ciphertext: uniform per cluster
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const bool xform = warp < L;  // warp-uniform
    const int lvl = xform ? warp : 0;
    const int tt = (warp & 1) * 32 + lane;  // warps 0, 1: thread of the inverse team
    const bool issuer = tid == NT - 32;  // lane 0 of the last warp, which runs no transform
    const Chan ch = pick_chan(a.ch, c);
    const uint2* inv16 = a.tw16 + (size_t)c * N;
    const uint64_t keep = l2_evict_last_policy();
    const uint32_t pinv = 0u - ch.pinv_neg;
    const uint32_t one_s = 0xFFFFFFFFu / ch.p;  // floor(2^32 / p): Shoup reduction by 1

    uint32_t* regions = reinterpret_cast<uint32_t*>(smem);          // [L][TBUF] transposes
    uint32_t* psum = regions + (size_t)L * Sh::TBUF;                // [N] the levels' partials, summed
    uint32_t* exch = psum + N;                                      // [2][L][N] written by the partner
    uint32_t* inbox = exch + (size_t)2 * L * N;                     // [2][3][N] row h's residues by channel
    int32_t* acc = reinterpret_cast<int32_t*>(inbox + 6 * N);       // [N] row h
    int16_t* dig = reinterpret_cast<int16_t*>(acc + N);             // [L][N]
    int16_t* sa = dig + (size_t)L * N;                              // [n+1]
    uint32_t* tab0 = reinterpret_cast<uint32_t*>((reinterpret_cast<uintptr_t>(sa + n + 1) + 3) & ~(uintptr_t)3);
    uint32_t* stage = reinterpret_cast<uint32_t*>(smem + brc6_stage_offset(n, L));  // [L][2][1024]
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + brc6_bars_offset(n, L));
    volatile int* stage_ok = reinterpret_cast<volatile int*>(bars + kCluster6Bars);
    uint32_t* sendbuf = reinterpret_cast<uint32_t*>(smem + brc6_send_offset(n, L));  // [2][L][N]
    const uint32_t bars_a = (uint32_t)__cvta_generic_to_shared(bars);
    const uint32_t tma_bar = bars_a;                                  // the key stage
    const uint32_t xbar0 = bars_a + 8u * (1 + lvl), xbar1 = xbar0 + 8u * kClusterMaxLevels;  // exchange, buffer 0/1
    const uint32_t ibar0 = bars_a + 8u * (1 + 2 * kClusterMaxLevels), ibar1 = ibar0 + 8u;    // inbox, buffer 0/1
    uint32_t* mine = regions + (size_t)lvl * Sh::TBUF;
    // the partner's exchange region of this level (buffer 0) and its barriers; the row peers'
    // inbox of channel c (buffer 0) and theirs
    const int partner = 3 * (1 - h) + c;
    const int peer_a = 3 * h + (c == 2 ? 0 : c + 1), peer_b = 3 * h + (c == 0 ? 2 : c - 1);
    const uint32_t x_dst = cluster_addr((uint32_t)__cvta_generic_to_shared(exch + (size_t)lvl * N), partner);
    const uint32_t x_bar0 = cluster_addr(xbar0, partner);  // buffer 1: + 8 kClusterMaxLevels
    const uint32_t box_local = (uint32_t)__cvta_generic_to_shared(inbox + (size_t)c * N);
    const uint32_t a_dst = cluster_addr(box_local, peer_a), b_dst = cluster_addr(box_local, peer_b);
    const uint32_t a_bar0 = cluster_addr(ibar0, peer_a), b_bar0 = cluster_addr(ibar0, peer_b);  // buffer 1: + 8

    const uint4* key = !valid ? nullptr : (a.key_of ? a.key_table[a.key_of[ct]] : a.key);
    const int64_t* lut = !valid ? nullptr : (a.lut_of ? a.lut_table[a.lut_of[ct]] : a.lut);
    bool tma = valid;  // uniform in the cluster
    if (tid == 0) {
        mbar_init(tma_bar, 1);
        for (int bb = 0; bb < 2; ++bb) {
            for (int lv = 0; lv < L; ++lv) mbar_init(bars_a + 8u * (1 + bb * kClusterMaxLevels + lv), 1);
            mbar_init(ibar0 + 8u * bb, 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // the issuer: arms the stage's barrier and copies the key rows of `step` (output h, channel c)
    auto issue = [&](int step) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(tma_bar, (uint32_t)L * 2 * 4096);
        for (int lv = 0; lv < L; ++lv)
            for (int row = 0; row < 2; ++row) {
                const size_t blk = (size_t)step * L + lv;
                const uint4* src = key + ((blk * 2 + row) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
                bulk_copy_g2s((uint32_t)__cvta_generic_to_shared(stage + (lv * 2 + row) * 1024), src, 4096, tma_bar);
            }
    };
    auto next_active = [&](int from) {
        while (from < a.steps && sa[from] == 0) ++from;
        return from;
    };
    uint32_t phase = 0;        // the issuer: parity of the stage's next barrier phase
    bool outstanding = false;  // the issuer: a copy whose wait gave up
    const bool use_tab0 = a.radix_bits <= 7;
    if (use_tab0) {
        for (int idx = tid; idx < 129; idx += NT) {
            const int d = idx - 64;
            const int64_t v = (int64_t)c_tw_head[PS][0][c][0][1].x * d % ch.p;
            tab0[64 + d] = (uint32_t)(v < 0 ? v + ch.p : v);
        }
    }
    if (valid) {
        if (a.scaled_in) {
            for (int i = tid; i < n; i += NT) sa[i] = (int16_t)a.scaled_in[(size_t)ct * n + i];
        } else {
            const int32_t* in = a.lwe_in + (size_t)ct * (n + 1);
            for (int i = tid; i <= n; i += NT) sa[i] = (int16_t)modswitch_down(in[i], 31 - 10, 11);
        }
    } else {
        for (int i = tid; i <= n; i += NT) sa[i] = 0;
    }
    for (int j = tid; j < N; j += NT) psum[j] = 0;
    __syncthreads();
    // the issuer copies the key rows of the next active step and waits for them (bounded)
    // while the transform warps work; stage_ok tells the step's readers whether they arrived
    auto refill = [&](int from) {
        const int f = next_active(from);
        if (!tma || f >= a.steps) return;
        issue(f);
        if (mbar_wait_bounded(tma_bar, phase, kWaitCycles)) {
            phase ^= 1;
            *stage_ok = 1;
        } else {
            atomicAdd(&g_wait_timeouts, 1ull);
            tma = false;  // read the key from global memory from here on
            outstanding = true;
            *stage_ok = 0;
        }
    };
    if (issuer) {
        *stage_ok = 0;
        refill(0);
    }
    if (valid && a.acc_in) {
        for (int j = tid; j < N; j += NT) acc[j] = (int32_t)a.acc_in[(size_t)ct * 2 * N + h * N + j];
    } else if (valid) {
        // genNoiselessTrlweSample: acc = (0, X^-b v) (yatfhe/src/trlwe.cpp:175-182)
        int t2 = -(int)sa[n];
        t2 = ((t2 % (2 * N)) + 2 * N) % (2 * N);
        const bool wrap = t2 >= N;
        const int at = wrap ? t2 - N : t2;
        for (int j = tid; j < N; j += NT) {
            int32_t v = j < at ? tneg<T>((int32_t)lut[j - at + N]) : (int32_t)lut[j - at];
            acc[j] = h == 0 ? 0 : (wrap ? tneg<T>(v) : v);
        }
    } else {
        for (int j = tid; j < N; j += NT) acc[j] = 0;
    }
    cluster.sync();  // every CTA has started and initialised its barriers

    int u = 0;          // active steps so far: buffer u & 1, barrier parity (u >> 1) & 1
    bool lost = false;  // a wait for another CTA gave up: stop waiting (the results are wrong, counted)
    for (int i = 0; i < a.steps; ++i) {
        const int ai = (int)sa[i];
        if (ai == 0) continue;  // the a_i = 0 skip (blind_rotate.cpp:1557), the same in every CTA
        const int t2 = ai < 0 ? ai + 2 * N : ai;
        const bool wrap = t2 >= N;
        const int at = wrap ? t2 - N : t2;
        const int b = u & 1;
        const uint32_t par = (uint32_t)(u >> 1) & 1u;
        ++u;
        // arm this step's barriers (their previous phases completed two active steps ago):
        // the partner's transform of each level, the row peers' residues
        if (xform && lane == 0) mbar_expect_tx(b ? xbar1 : xbar0, 4096);  // one arrival per phase
        if (issuer) mbar_expect_tx(b ? ibar1 : ibar0, 2 * 4096);
        // (1) X^{a_i} row - row, zero-mean digits (rotateTrlweMinusOne, gadgetDecomposeTrlwe)
        auto decompose = [&](auto lc, auto rc) {
            constexpr int LC = decltype(lc)::value, RC = decltype(rc)::value;
            const int levels = LC ? LC : L, radix = RC ? RC : a.radix_bits;
            // coefficients tid + e NT: every accumulator word is loaded before any digit is stored
            constexpr int E = N / NT;
            int32_t tmp[E];
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int j = tid + e * NT;
                int32_t rot = j < at ? tneg<T>(acc[j - at + N]) : acc[j - at];
                if (wrap) rot = tneg<T>(rot);
                tmp[e] = tsub<T>(rot, acc[j]);
            }
#pragma unroll
            for (int e = 0; e < E; ++e) {
                int16_t* d = dig + tid + e * NT;
                zero_mean_digits<uint32_t, 32>((uint32_t)tmp[e], levels, radix, [&](int level, int v) { d[level * N] = (int16_t)v; });
            }
        };
        if (L == 3 && a.radix_bits == 7)
            decompose(std::integral_constant<int, 3>{}, std::integral_constant<int, 7>{});
        else
            decompose(std::integral_constant<int, 0>{}, std::integral_constant<int, 0>{});
        __syncthreads();
        if (xform) {
            // (2) this level's forward transform, stored into the partner's exchange region
            uint32_t x[32];
            const int16_t* d = dig + (size_t)lvl * N;
            if (use_tab0) {
#pragma unroll
                for (int r = 0; r < 32; ++r) x[r] = (uint32_t)(int32_t)d[r * S + lane];
                ntt_forward<10, PS, 1>(x, mine, lane, c, 0, ch, tab0 + 64);
            } else {
                const uint32_t bias = fwd_bias_digits<10, PS>(ch.p);
#pragma unroll
                for (int r = 0; r < 32; ++r) x[r] = (uint32_t)(int32_t)d[r * S + lane] + bias;
                ntt_forward<10, PS>(x, mine, lane, c, 0, ch);
            }
            {
                const uint32_t dst = x_dst + 4u * (uint32_t)(b * L * N), bar = x_bar0 + 8u * kClusterMaxLevels * b;
                uint32_t* sb = sendbuf + ((size_t)b * L + lvl) * N;
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    *reinterpret_cast<uint4*>(sb + swz(lane, k)) = make_uint4(x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3]);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) bulk_s2c(dst, (uint32_t)__cvta_generic_to_shared(sb), 4096, bar);
            }
            // the helper warp (4 + lvl) takes slots 16..31 of each lane: it may read the send buffer
            asm volatile("bar.arrive %0, 64;" ::"r"(2 + lvl) : "memory");
            // own row with K(lvl, h, h) while the partner finishes: x < 46p and key words < p,
            // so the sum of two products fits 64 bits
            const size_t blk = (size_t)i * L + lvl;
            const uint4* gown = key + ((blk * 2 + h) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
            const uint4* gpar = key + ((blk * 2 + (1 - h)) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
            const bool from_stage = *stage_ok;
            const uint32_t* theirs = exch + ((size_t)b * L + lvl) * N;
            {
                const uint4* kown = from_stage ? reinterpret_cast<const uint4*>(stage + (lvl * 2 + h) * 1024) : nullptr;
                const uint4* spar = from_stage ? reinterpret_cast<const uint4*>(stage + (lvl * 2 + (1 - h)) * 1024) : nullptr;
                uint64_t own[16];
#pragma unroll
                for (int rr = 0; rr < 4; ++rr) {
                    const uint4 ka = from_stage ? kown[rr * S + lane] : ldg_keep(gown + rr * S + lane, keep);
                    const uint32_t kav[4] = {ka.x, ka.y, ka.z, ka.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) own[rr * 4 + e] = (uint64_t)x[rr * 4 + e] * kav[e];
                }
                if (!lost && !mbar_wait_cluster_bounded(b ? xbar1 : xbar0, par, kWaitCycles)) {
                    lost = true;
                    atomicAdd(&g_wait_timeouts, 1ull);
                }
                // (3) the partner's row with K(lvl, 1 - h, h), one Montgomery reduction per sum;
                // the partials are stored after every load, so the loads need not wait for them
                uint32_t res[16];
#pragma unroll
                for (int rr = 0; rr < 4; ++rr) {
                    const uint4 kb = from_stage ? spar[rr * S + lane] : ldg_keep(gpar + rr * S + lane, keep);
                    const uint4 tb = *reinterpret_cast<const uint4*>(theirs + swz(lane, rr));
                    const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w}, tv[4] = {tb.x, tb.y, tb.z, tb.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int r = rr * 4 + e;
                        const uint64_t s = own[r] + (uint64_t)tv[e] * kbv[e];
                        // s 2^-32 mod p (Montgomery) + p: in (0, 3.1p), reduced after the level sum
                        res[r] = (uint32_t)(s >> 32) - __umulhi((uint32_t)s * pinv, ch.p) + ch.p;
                    }
                }
#pragma unroll
                for (int r = 0; r < 16; ++r) atomicAdd(&psum[r * S + lane], res[r]);
            }
        } else if (warp >= 4 && warp - 4 < L) {
            // helper of level hl: slots 16..31 of each lane, its transform read from the send buffer
            const int hl = warp - 4;
            asm volatile("bar.sync %0, 64;" ::"r"(2 + hl) : "memory");
            const uint32_t* sb = sendbuf + ((size_t)b * L + hl) * N;
            const size_t blk = (size_t)i * L + hl;
            const uint4* gown = key + ((blk * 2 + h) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
            const uint4* gpar = key + ((blk * 2 + (1 - h)) * kChannels + c) * (key_block_words(N) / 4) + (h ? 8 : 0) * S;
            const bool from_stage = *stage_ok;
            const uint32_t* theirs = exch + ((size_t)b * L + hl) * N;
            const uint4* kown = from_stage ? reinterpret_cast<const uint4*>(stage + (hl * 2 + h) * 1024) : nullptr;
            const uint4* spar = from_stage ? reinterpret_cast<const uint4*>(stage + (hl * 2 + (1 - h)) * 1024) : nullptr;
            uint64_t own[16];
#pragma unroll
            for (int rr = 4; rr < 8; ++rr) {
                const uint4 xa = *reinterpret_cast<const uint4*>(sb + swz(lane, rr));
                const uint4 ka = from_stage ? kown[rr * S + lane] : ldg_keep(gown + rr * S + lane, keep);
                own[(rr - 4) * 4 + 0] = (uint64_t)xa.x * ka.x;
                own[(rr - 4) * 4 + 1] = (uint64_t)xa.y * ka.y;
                own[(rr - 4) * 4 + 2] = (uint64_t)xa.z * ka.z;
                own[(rr - 4) * 4 + 3] = (uint64_t)xa.w * ka.w;
            }
            const uint32_t hbar = bars_a + 8u * (1 + b * kClusterMaxLevels + hl);
            if (!lost && !mbar_wait_cluster_bounded(hbar, par, kWaitCycles)) {
                lost = true;
                atomicAdd(&g_wait_timeouts, 1ull);
            }
            uint32_t res[16];
#pragma unroll
            for (int rr = 4; rr < 8; ++rr) {
                const uint4 kb = from_stage ? spar[rr * S + lane] : ldg_keep(gpar + rr * S + lane, keep);
                const uint4 tb = *reinterpret_cast<const uint4*>(theirs + swz(lane, rr));
                const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w}, tv[4] = {tb.x, tb.y, tb.z, tb.w};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int q = (rr - 4) * 4 + e;
                    const uint64_t s = own[q] + (uint64_t)tv[e] * kbv[e];
                    res[q] = (uint32_t)(s >> 32) - __umulhi((uint32_t)s * pinv, ch.p) + ch.p;
                }
            }
#pragma unroll
            for (int q = 0; q < 16; ++q) atomicAdd(&psum[(16 + q) * S + lane], res[q]);
        }
        __syncthreads();  // every partial is in, and the stage has been read
        if (issuer) refill(i + 1);
        // (4) warps 0 and 1: sum of the l partials, inverse transform, residues to the row's CTAs
        if (warp < 2) {
            uint32_t oa[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                // slot s of register q of thread tt: its partial sum sits at (s mod 32) 32 + s / 32
                const int sl = slot16(tt, q);
                const uint32_t v = psum[(sl & 31) * 32 + (sl >> 5)];
                oa[q] = v - __umulhi(v, one_s) * ch.p;  // l terms < 3.1p each: < 13p; reduced to [0, 2p)
            }
            ntt16_inverse(oa, regions, tt, 0, ch, inv16);  // transposes in warp 0's region, after every partial was read
            uint32_t* box = inbox + ((size_t)b * 3 + c) * N;
            const uint32_t off = 4u * (uint32_t)(b * 3 * N);
            const uint32_t abar = a_bar0 + 8u * b, bbar = b_bar0 + 8u * b;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint4 v = make_uint4(reduce_once(oa[4 * k], ch.p), reduce_once(oa[4 * k + 1], ch.p),
                                           reduce_once(oa[4 * k + 2], ch.p), reduce_once(oa[4 * k + 3], ch.p));
                *reinterpret_cast<uint4*>(box + swz16(tt, k)) = v;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            team16_sync(0);
            if (tt == 0) {
                const uint32_t src = (uint32_t)__cvta_generic_to_shared(box);
                bulk_s2c(a_dst + off, src, 4096, abar);
                bulk_s2c(b_dst + off, src, 4096, bbar);
            }
        }
        __syncthreads();  // this channel's residues are in the inbox
        if (!lost && !mbar_wait_cluster_bounded(b ? ibar1 : ibar0, par, kWaitCycles)) {
            lost = true;
            atomicAdd(&g_wait_timeouts, 1ull);
        }
        // (5) CRT -> applyIntt's centred mod-q value mod 2^32, accumulateTrlwe on row h: this
        // thread's chunk, chunk tid >> 6 of inverse-team thread tid & 63, coefficients
        // (4 (tid >> 6) + e) 64 + (tid & 63)
        *reinterpret_cast<uint4*>(psum + 4 * tid) = make_uint4(0, 0, 0, 0);  // read before the inbox barrier
        {
            const int ck = tid >> 6, cl = tid & 63;
            const uint32_t* box = inbox + (size_t)b * 3 * N + swz16(cl, ck);
            const uint4 r0 = *reinterpret_cast<const uint4*>(box);
            const uint4 r1 = *reinterpret_cast<const uint4*>(box + N);
            const uint4 r2 = *reinterpret_cast<const uint4*>(box + 2 * N);
            const uint32_t v0[4] = {r0.x, r0.y, r0.z, r0.w}, v1[4] = {r1.x, r1.y, r1.z, r1.w}, v2[4] = {r2.x, r2.y, r2.z, r2.w};
            uint32_t old[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) old[e] = (uint32_t)acc[(4 * ck + e) * 64 + cl];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int64_t v = crt_to_torus<T>(v0[e], v1[e], v2[e], a.crt);
                acc[(4 * ck + e) * 64 + cl] = (int32_t)(old[e] + (uint32_t)v);
            }
        }
        __syncthreads();
    }

    if (valid && a.acc_out && c == 0) {
        int64_t* dst = a.acc_out + (size_t)ct * 2 * N + h * N;
        for (int j = tid; j < N; j += NT) dst[j] = (int64_t)acc[j];
    }
    if (valid && a.big_out && c == 0) {
        // extractTlweFromTrlwe(out, acc, 0): a'[j] = j ? -a[N-j] : a[0] from row 0, b' = b[0] from row 1
        int32_t* dst = a.big_out + (size_t)ct * (N + 1);
        if (h == 0) {
            for (int j = tid; j < N; j += NT) dst[j] = j == 0 ? acc[0] : tneg<T>(acc[N - j]);
        } else if (tid == 0) {
            dst[N] = acc[0];
        }
    }
    // a copy whose wait gave up may still land: wait for it (bounded) before the CTA exits
    if (outstanding && issuer && !mbar_wait_bounded(tma_bar, phase, kWaitCycles)) atomicAdd(&g_wait_timeouts, 1ull);
    cluster.sync();  // no CTA leaves while another may still store into its regions
}

constexpr int kKsTile = kKsTileCts;  // ciphertexts per block of multi-key and small batches
constexpr int kKsTileWide = 32;      // ciphertexts per block of large single-key batches
constexpr int kKsCols = 128;    // output columns per block (= threads)
constexpr int kKsChunk = 32;    // input coefficients per digit refresh
constexpr int kKsMaxT = 16;
constexpr int kKsSplitCtasPerSm = 4;  // small batches: split the input until the grid has this many per SM
constexpr int kKsMinSplitCoefs = 8;   // input coefficients of one split at least

// Tiles of ciphertexts x output columns.  For small batches the input coefficients are also
// split across gridDim.z CTAs (the grid would otherwise be a few CTAs, each streaming its
// share of the whole key at one thread's memory parallelism): each adds its partial sum into
// the zeroed output with atomic 32-bit adds, which wrap mod 2^32 like the sum itself, so the
// result does not depend on their order.  TILE ciphertexts share each key word a thread
// loads: 32 for large single-key batches (the key is read from L2 a quarter as often as with
// 8: 38.2 against 42.3 ms at 65,536 ciphertexts, T32), 8 for multi-key tiles and small batches,
// whose tiles are often not full.
template <int TILE>
__global__ void __launch_bounds__(kKsCols) keyswitch_kernel(const KsArgs a) {
    __shared__ int8_t sdig[TILE][kKsChunk][kKsMaxT];
    __shared__ int32_t sb[TILE];
    const int x = blockIdx.y * kKsCols + threadIdx.x;
    const int splits = (int)gridDim.z;
    const int per = (a.kN + splits - 1) / splits;
    const int i_begin = (int)blockIdx.z * per, i_end = min(a.kN, i_begin + per);
    int c0, cnt;
    const int32_t* ksk;
    if (a.tiles) {
        const KsTile tl = a.tiles[blockIdx.x];
        c0 = tl.ct_begin;
        cnt = tl.count;
        ksk = tl.ksk;
    } else {
        c0 = blockIdx.x * TILE;
        cnt = min(TILE, a.count - c0);
        ksk = a.ksk;
    }
    const int nb = a.n + 1;
    uint32_t acc[TILE];
#pragma unroll
    for (int c = 0; c < TILE; ++c) acc[c] = 0;
    if (threadIdx.x < TILE) {
        const int ct = c0 + threadIdx.x;
        sb[threadIdx.x] = (int)threadIdx.x < cnt ? a.big_in[(size_t)ct * (a.kN + 1) + a.kN] : 0;
    }
    for (int i0 = i_begin; i0 < i_end; i0 += kKsChunk) {
        __syncthreads();
        for (int e = threadIdx.x; e < TILE * kKsChunk; e += kKsCols) {
            const int c = e / kKsChunk, ii = e % kKsChunk;
            const int ct = c0 + c, i = i0 + ii;
            const int32_t v = (c < cnt && i < i_end) ? a.big_in[(size_t)ct * (a.kN + 1) + i] : 0;
            zero_mean_digits<uint32_t, 32>((uint32_t)v, a.t, a.ks_radix_bits,
                                           [&](int level, int d) { sdig[c][ii][level] = (int8_t)d; });
        }
        __syncthreads();
        if (x < nb) {
            const int iend = min(kKsChunk, i_end - i0);
            for (int ii = 0; ii < iend; ++ii) {
                const int32_t* row = ksk + ((size_t)(i0 + ii) * a.t) * nb + x;
                for (int j = 0; j < a.t; ++j) {
                    const uint32_t w = (uint32_t)__ldg(row + (size_t)j * nb);
#pragma unroll
                    for (int c = 0; c < TILE; ++c) acc[c] += (uint32_t)(int32_t)sdig[c][ii][j] * w;
                }
            }
        }
    }
    if (x < nb) {
#pragma unroll
        for (int c = 0; c < TILE; ++c) {
            const int ct = c0 + c;
            if (c >= cnt) continue;
            const uint32_t v = (x == a.n && blockIdx.z == 0 ? (uint32_t)sb[c] : 0u) - acc[c];
            if (splits == 1) a.out[(size_t)ct * nb + x] = (int32_t)v;
            else atomicAdd(reinterpret_cast<unsigned int*>(a.out + (size_t)ct * nb + x), v);
        }
    }
}

template <int LOGN, int T, int G, int SPLIT>
int prepare_br_t() {
    // the dynamic shared-memory opt-in is per device: done once on each
    static std::atomic<bool> done[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
    if (!done[dev].load()) {
        if (cudaFuncSetAttribute(blind_rotate_kernel<LOGN, T, G, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 227 * 1024) != cudaSuccess)
            return -1;
        done[dev].store(true);
    }
    return 0;
}

template <int LOGN, int T, int G, int SPLIT>
int launch_br_t(const BrArgs& a, void* stream) {
    const size_t smem = (size_t)G * br_smem_bytes(LOGN, T, a.n, a.L, SPLIT);
    if (smem > 227 * 1024) return -1;
    if (prepare_br_t<LOGN, T, G, SPLIT>() != 0) return -1;
    const int need = (a.count + G - 1) / G;
    const int grid = a.grid > 0 && a.grid < need ? a.grid : need;
    blind_rotate_kernel<LOGN, T, G, SPLIT>
        <<<grid, G * slice_threads<LOGN, SPLIT>(), smem, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int LOGN, int T, int G, int SPLIT>
int ctas_per_sm_t(int n, int L) {
    const size_t smem = (size_t)G * br_smem_bytes(LOGN, T, n, L, SPLIT);
    if (smem > 227 * 1024) return 0;
    if (prepare_br_t<LOGN, T, G, SPLIT>() != 0) return -1;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, blind_rotate_kernel<LOGN, T, G, SPLIT>,
                                                      G * slice_threads<LOGN, SPLIT>(), smem) != cudaSuccess)
        return -1;
    return blocks;
}

struct LaunchBr {
    const BrArgs& a;
    void* stream;
    template <int LN, int TB, int GG, int SP>
    int operator()() const { return launch_br_t<LN, TB, GG, SP>(a, stream); }
};

struct OccupancyBr {
    int n, L;
    template <int LN, int TB, int GG, int SP>
    int operator()() const { return ctas_per_sm_t<LN, TB, GG, SP>(n, L); }
};

// Dispatch on (N, torus width, ciphertexts per CTA, layout); F(tag) gets the template
// arguments.  kNoVariant when that combination is not compiled.
template <typename F>
int dispatch_br(int logN, int torus_bits, int g, int layout, F&& f) {
    if (g <= 0) g = 1;
#define YG_BR_CASE(LN, TB, GG, SP)                                                          \
    if (logN == LN && torus_bits == TB && g == GG && layout == SP)                          \
        return f.template operator()<LN, TB, GG, SP>();
    YG_BR_CASE(10, 32, 1, 0) YG_BR_CASE(10, 32, 2, 0) YG_BR_CASE(10, 32, 4, 0)
    YG_BR_CASE(10, 56, 1, 0) YG_BR_CASE(10, 56, 2, 0) YG_BR_CASE(10, 56, 4, 0)
    YG_BR_CASE(11, 32, 1, 0) YG_BR_CASE(11, 32, 2, 0)
    YG_BR_CASE(11, 56, 1, 0) YG_BR_CASE(11, 56, 2, 0)
    YG_BR_CASE(10, 32, 1, 1) YG_BR_CASE(10, 32, 2, 1)
    YG_BR_CASE(10, 56, 1, 1) YG_BR_CASE(10, 56, 2, 1)
    YG_BR_CASE(11, 32, 1, 1) YG_BR_CASE(11, 56, 1, 1)
#undef YG_BR_CASE
    return kNoVariant;
}

}  // namespace


int set_twiddle_heads(int logN, int ps, const uint2* heads) {
    if ((logN != 10 && logN != 11) || ps < 0 || ps >= kPrimeSets) return -1;
    const size_t per = sizeof(uint2) * kChannels * 2 * 32;
    return cudaMemcpyToSymbol(c_tw_head, heads, per, per * (ps * 2 + logN - 10)) == cudaSuccess ? 0 : -1;
}

int launch_keyconv(int logN, int ps, const KeyConvArgs& a, void* stream) {
    const dim3 grid(a.polys);
    if (logN == 10 && ps == 0) keyconv_kernel<10, 0><<<grid, 3 * TeamShape<10>::S, 0, (cudaStream_t)stream>>>(a);
    else if (logN == 10 && ps == 1) keyconv_kernel<10, 1><<<grid, 3 * TeamShape<10>::S, 0, (cudaStream_t)stream>>>(a);
    else if (logN == 11 && ps == 0) keyconv_kernel<11, 0><<<grid, 3 * TeamShape<11>::S, 0, (cudaStream_t)stream>>>(a);
    else if (logN == 11 && ps == 1) keyconv_kernel<11, 1><<<grid, 3 * TeamShape<11>::S, 0, (cudaStream_t)stream>>>(a);
    else return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

namespace {

// The cluster kernels exist for T = 32, N = 1024, one ciphertext per cluster, l <= 4.
bool cluster_variant(int logN, int torus_bits, int per_cta, int L) {
    return logN == 10 && torus_bits == 32 && per_cta <= 1 && L >= 1 && L <= kClusterMaxLevels;
}

int prepare_brc() {
    static std::atomic<bool> done[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
    if (!done[dev].load()) {
        if (cudaFuncSetAttribute(blind_rotate_cluster_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 227 * 1024) != cudaSuccess ||
            cudaFuncSetAttribute(blind_rotate_cluster6_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 227 * 1024) != cudaSuccess)
            return -1;
        done[dev].store(true);
    }
    return 0;
}

}  // namespace

int launch_blind_rotate(int logN, int torus_bits, const BrArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    if (a.layout == kLayoutRowCluster) {
        if (!cluster_variant(logN, torus_bits, a.per_cta, a.L)) return kNoVariant;
        const size_t smem = brc_smem_bytes(a.n, a.L);
        if (smem > 227 * 1024 || prepare_brc() != 0) return -1;
        blind_rotate_cluster_kernel<32><<<2 * a.count, kChannels * a.L * 32, smem, (cudaStream_t)stream>>>(a);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    }
    if (a.layout == kLayoutChannelCluster) {
        if (!cluster_variant(logN, torus_bits, a.per_cta, a.L)) return kNoVariant;
        const size_t smem = brc6_smem_bytes(a.n, a.L);
        if (smem > 227 * 1024 || prepare_brc() != 0) return -1;
        if (!a.tw16) return -1;  // the 16-residue inverse's tables (built for every T = 32, N = 1024 context)
        blind_rotate_cluster6_kernel<32><<<6 * a.count, kCluster6Warps * 32, smem, (cudaStream_t)stream>>>(a);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    }
    return dispatch_br(logN, torus_bits, a.per_cta, a.layout, LaunchBr{a, stream});
}

int br_ctas_per_sm(int logN, int torus_bits, int n, int L, int per_cta, int layout) {
    if (layout == kLayoutRowCluster) {
        if (!cluster_variant(logN, torus_bits, per_cta, L)) return 0;
        const size_t smem = brc_smem_bytes(n, L);
        if (smem > 227 * 1024) return 0;
        if (prepare_brc() != 0) return -1;
        int blocks = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, blind_rotate_cluster_kernel<32>, kChannels * L * 32,
                                                          smem) != cudaSuccess) {
            // the calculator may decline cluster kernels: its shared memory fits and 168
            // registers x 3 l warps (l <= 4) fit one SM's register file
            (void)cudaGetLastError();
            blocks = 1;
        }
        return blocks;
    }
    if (layout == kLayoutChannelCluster) {
        if (!cluster_variant(logN, torus_bits, per_cta, L)) return 0;
        const size_t smem = brc6_smem_bytes(n, L);
        if (smem > 227 * 1024) return 0;
        if (prepare_brc() != 0) return -1;
        int blocks = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, blind_rotate_cluster6_kernel<32>, kCluster6Warps * 32,
                                                          smem) != cudaSuccess) {
            // the calculator may decline cluster kernels: 168 registers x 256 threads and the
            // shared memory fit one SM
            (void)cudaGetLastError();
            blocks = 1;
        }
        return blocks;
    }
    return dispatch_br(logN, torus_bits, per_cta, layout, OccupancyBr{n, L});
}

int cluster6_max_clusters(int n, int L) {
    if (L < 1 || L > kClusterMaxLevels || brc6_smem_bytes(n, L) > 227 * 1024 || prepare_brc() != 0) return 0;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(6);
    cfg.blockDim = dim3(kCluster6Warps * 32);
    cfg.dynamicSmemBytes = brc6_smem_bytes(n, L);
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, blind_rotate_cluster6_kernel<32>, &cfg) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return clusters;
}

int launch_key_intt(const KeyInttArgs& a, void* stream) {
    if (a.polys <= 0) return 0;
    if (a.N != 1024 && a.N != 2048) return -1;
    key_intt_kernel<<<a.polys, a.N / 2, (size_t)a.N * sizeof(uint64_t), (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_wwl24_expand(const WwlExpandArgs& a, void* stream) {
    if (a.n <= 0) return 0;
    if ((a.N != 1024 && a.N != 2048) || a.L < 1 || a.Ls < 1 || a.Ls > kWwlMaxLevels) return -1;
    const size_t smem = (size_t)a.N * sizeof(uint64_t);
    if (a.torus_bits == 32)
        wwl24_expand_kernel<32><<<a.n * a.L, a.N / 2, smem, (cudaStream_t)stream>>>(a);
    else if (a.torus_bits == 56)
        wwl24_expand_kernel<56><<<a.n * a.L, a.N / 2, smem, (cudaStream_t)stream>>>(a);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_keygen_bsk(const KeygenBskArgs& a, void* stream) {
    if (a.n <= 0) return 0;
    if ((a.N != 1024 && a.N != 2048) || a.k != 1 || a.L < 1) return -1;
    const int blocks = a.n * a.L * (a.k + 1);
    const size_t smem = (size_t)a.N * sizeof(uint64_t);
    if (a.torus_bits == 32)
        keygen_bsk_kernel<32><<<blocks, a.N / 2, smem, (cudaStream_t)stream>>>(a);
    else if (a.torus_bits == 56)
        keygen_bsk_kernel<56><<<blocks, a.N / 2, smem, (cudaStream_t)stream>>>(a);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_encrypt_rlwe_ntt(const EncryptRlweArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    if ((a.N != 1024 && a.N != 2048) || a.k != 1 || a.ctas < 1) return -1;
    const size_t smem = (size_t)(a.k + 1) * a.N * sizeof(uint64_t);
    const int grid = a.count < a.ctas ? a.count : a.ctas;
    if (a.torus_bits == 32)
        encrypt_rlwe_ntt_kernel<32><<<grid, a.N / 2, smem, (cudaStream_t)stream>>>(a);
    else if (a.torus_bits == 56)
        encrypt_rlwe_ntt_kernel<56><<<grid, a.N / 2, smem, (cudaStream_t)stream>>>(a);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_keygen_ksk(const KeygenKskArgs& a, void* stream) {
    const long samples = (long)a.kN * a.t;
    if (samples <= 0) return 0;
    if (a.ks_radix_bits < 1 || a.t * a.ks_radix_bits > 32) return -1;
    keygen_ksk_kernel<<<(unsigned)((samples + 7) / 8), 256, 0, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_lazy_blind_rotate(const LazyBrArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    if ((a.N != 1024 && a.N != 2048) || a.n < 2 || a.L < 1 || a.L > kLazyMaxLevels || a.Ls < 1 ||
        a.Ls > kLazyMaxLevels)
        return -1;
    const size_t smem = lazy_br_smem_bytes(a.N, a.torus_bits, a.n, a.L, a.Ls);
    auto go = [&](auto kern) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
        kern<<<a.count, a.N / 2, smem, (cudaStream_t)stream>>>(a);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    };
    if (a.torus_bits == 32) return go(lazy_blind_rotate_kernel<32>);
    if (a.torus_bits == 56) return go(lazy_blind_rotate_kernel<56>);
    return -1;
}

int launch_group_blind_rotate(const GroupBrArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    if ((a.N != 1024 && a.N != 2048) || a.group < 1 || a.group > 3 || a.n % a.group || a.L < 1 ||
        a.L > a.l_full || a.l_full > kGroupMaxLevels || (!a.lut && !a.acc_in) || (!a.lwe_in && !a.scaled_in) ||
        (a.scaled_in && !a.acc_in))
        return -1;
    const size_t smem = group_br_smem_bytes(a.N, a.torus_bits, a.n, a.L);
    auto go = [&](auto kern) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
        kern<<<a.count, a.N / 2, smem, (cudaStream_t)stream>>>(a);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    };
    if (a.torus_bits == 32) return go(group_blind_rotate_kernel<32>);
    if (a.torus_bits == 56) return go(group_blind_rotate_kernel<56>);
    return -1;
}

int read_wait_timeouts(unsigned long long* out) {
    return cudaMemcpyFromSymbol(out, g_wait_timeouts, sizeof(*out)) == cudaSuccess ? 0 : -1;
}

int preload_keyswitch() {
    cudaFuncAttributes attr;
    return cudaFuncGetAttributes(&attr, keyswitch_kernel<kKsTile>) == cudaSuccess &&
                   cudaFuncGetAttributes(&attr, keyswitch_kernel<kKsTileWide>) == cudaSuccess
               ? 0
               : -1;
}

int launch_keyswitch(const KsArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    if (a.t > kKsMaxT) return -1;
    const int blocks = a.tiles ? a.num_tiles : (a.count + kKsTile - 1) / kKsTile;
    if (blocks <= 0) return 0;
    const int cols = (a.n + 1 + kKsCols - 1) / kKsCols;
    static std::atomic<int> sms[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
    int sm_count = sms[dev].load(std::memory_order_relaxed);
    if (sm_count == 0) {
        if (cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
        sms[dev].store(sm_count, std::memory_order_relaxed);
    }
    const long long want = (long long)kKsSplitCtasPerSm * sm_count;
    // a single-key batch whose grid of wide tiles still fills the GPU takes wide tiles
    if (!a.tiles) {
        const int wide = (a.count + kKsTileWide - 1) / kKsTileWide;
        if ((long long)wide * cols >= want) {
            keyswitch_kernel<kKsTileWide><<<dim3(wide, cols, 1), kKsCols, 0, (cudaStream_t)stream>>>(a);
            return cudaGetLastError() == cudaSuccess ? 0 : -1;
        }
    }
    // a grid of fewer than kKsSplitCtasPerSm CTAs per SM splits the input coefficients (at
    // least kKsMinSplitCoefs each) across CTAs that add into the zeroed output
    int splits = 1;
    if ((long long)blocks * cols < want) {
        const long long by_grid = (want + (long long)blocks * cols - 1) / ((long long)blocks * cols);
        splits = (int)std::min<long long>(by_grid, std::max(1, a.kN / kKsMinSplitCoefs));
        splits = (a.kN + (a.kN + splits - 1) / splits - 1) / ((a.kN + splits - 1) / splits);  // no empty split
    }
    if (splits > 1 &&
        cudaMemsetAsync(a.out, 0, (size_t)a.count * (a.n + 1) * sizeof(int32_t), (cudaStream_t)stream) != cudaSuccess)
        return -1;
    dim3 grid(blocks, cols, splits);
    keyswitch_kernel<kKsTile><<<grid, kKsCols, 0, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yg
