// pbs_kernels.cu -- GB300 kernels of the GINX/MP21 programmable bootstrap.
//
//   keyconv_kernel       BSK coefficient residues -> per-channel NTT, slot layout, Montgomery
//                        form with N^-1 folded in (done once per key upload)
//   blind_rotate_kernel  rescaleTlweToNewMod + genNoiselessTrlweSample + the MP21 CMux loop
//                        (yatfhe/src/blind_rotate.cpp:1538-1565) + extractTlweFromTrlwe
//                        (yatfhe/src/trlwe.cpp:240-250); one CTA per ciphertext, its
//                        accumulator resident in shared memory for all n steps
//   keyswitch_kernel     switchKeyForTlwe (yatfhe/src/keyswitching.cpp:48-72) for a tile of
//                        ciphertexts x output columns, KSK rows streamed once per tile
#include <cuda_runtime.h>

#include <type_traits>

#include "ntt.cuh"
#include "pbs_kernels.cuh"

namespace yg {

namespace {

__device__ __forceinline__ Chan pick_chan(const Chan (&c)[kChannels], int team) {
    return team == 0 ? c[0] : (team == 1 ? c[1] : c[2]);
}

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

template <int LOGN>
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
#pragma unroll
    for (int r = 0; r < 32; ++r) x[r] = src[r * S + tt];
    ntt_forward<LOGN>(x, tb + team * Sh::TBUF, tt, team, ch);
    const int blk = poly >> 1, o = poly & 1;
    uint32_t* dst = a.key + ((size_t)blk * kChannels + team) * key_block_words(N);
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        const uint32_t y = reduce_once(reduce_once(mulshoup(x[r], sc, scs, ch.p), ch.two_p), ch.p);
        dst[((o * 8 + (r >> 2)) * S + tt) * 4 + (r & 3)] = y;
    }
}

template <int LOGN, int T>
__global__ void __launch_bounds__(3 * TeamShape<LOGN>::S) blind_rotate_kernel(const BrArgs a) {
    using Sh = TeamShape<LOGN>;
    using TorusT = typename TorusOf<T>::type;
    using U = typename TorusOf<T>::utype;
    constexpr int N = Sh::N, S = Sh::S;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* tb = reinterpret_cast<uint32_t*>(smem);               // [3][TBUF] transposes
    uint32_t* xb = tb + kChannels * Sh::TBUF;                        // [3][2][N] INTT outputs
    TorusT* acc = reinterpret_cast<TorusT*>(xb + kChannels * 2 * N); // [2][N] accumulator
    int16_t* dig = reinterpret_cast<int16_t*>(acc + 2 * N);          // [2][L][N] digits
    int16_t* sa = dig + 2 * a.L * N;                                  // [n+1] mod-2N input

    const int ct = blockIdx.x;
    const int tid = threadIdx.x, nth = blockDim.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int team = warp / Sh::WARPS;
    const int tt = (warp % Sh::WARPS) * 32 + lane;
    const Chan ch = pick_chan(a.ch, team);
    const int L = a.L, n = a.n;

    // rescaleTlweToNewMod into mod 2N (yatfhe/src/tlwe.cpp:75-81), unless given already scaled
    if (a.scaled_in) {
        const int32_t* in = a.scaled_in + (size_t)ct * n;
        for (int i = tid; i < n; i += nth) sa[i] = (int16_t)in[i];
    } else {
        const int32_t* in = a.lwe_in + (size_t)ct * (n + 1);
        for (int i = tid; i <= n; i += nth) sa[i] = (int16_t)modswitch_down(in[i], 31 - LOGN, LOGN + 1);
    }
    __syncthreads();

    if (a.acc_in) {
        const int64_t* src = a.acc_in + (size_t)ct * 2 * N;
        for (int idx = tid; idx < 2 * N; idx += nth) acc[idx] = (TorusT)src[idx];
    } else {
        // genNoiselessTrlweSample: acc = (0, X^-b v) (yatfhe/src/trlwe.cpp:175-182)
        int t2 = -(int)sa[n];
        t2 = ((t2 % (2 * N)) + 2 * N) % (2 * N);
        const bool wrap = t2 >= N;
        const int at = wrap ? t2 - N : t2;
        for (int j = tid; j < N; j += nth) {
            acc[j] = 0;
            TorusT v = j < at ? tneg<T>((TorusT)a.lut[j - at + N]) : (TorusT)a.lut[j - at];
            acc[N + j] = wrap ? tneg<T>(v) : v;
        }
    }
    __syncthreads();

    for (int i = 0; i < a.steps; ++i) {
        const int ai = sa[i];
        if (ai == 0) continue;  // result-neutral skip of blind_rotate.cpp:1557
        // tmp = X^{a_i} acc - acc (rotateTrlweMinusOne, yatfhe/src/trlwe.cpp:284-289), then
        // gadgetDecomposeTrlwe (yatfhe/src/trlwe.cpp:185-198) into int16 digits
        {
            const int t2 = ai < 0 ? ai + 2 * N : ai;
            const bool wrap = t2 >= N;
            const int at = wrap ? t2 - N : t2;
            for (int idx = tid; idx < 2 * N; idx += nth) {
                const int o = idx >= N;
                const int j = idx - o * N;
                const TorusT* A = acc + o * N;
                TorusT rot = j < at ? tneg<T>(A[j - at + N]) : A[j - at];
                if (wrap) rot = tneg<T>(rot);
                const TorusT tmp = tsub<T>(rot, A[j]);
                int16_t* d = dig + (size_t)o * L * N + j;
                zero_mean_digits<U, T>((U)tmp, L, a.radix_bits,
                                       [&](int level, int v) { d[(size_t)level * N] = (int16_t)v; });
            }
        }
        __syncthreads();

        // externalProductTrgswMPNttImpl (yatfhe/src/trgsw.cpp:712-767) in channel `team`:
        // forward NTT of every digit poly, Montgomery MAC against the key, inverse NTT.
        uint32_t oa[32], ob[32];
#pragma unroll
        for (int r = 0; r < 32; ++r) oa[r] = ob[r] = 0;
        for (int row = 0; row < 2; ++row) {
            for (int lvl = 0; lvl < L; ++lvl) {
                uint32_t x[32];
                const int16_t* d = dig + ((size_t)row * L + lvl) * N;
#pragma unroll
                for (int r = 0; r < 32; ++r) x[r] = (uint32_t)((int32_t)d[r * S + tt] + (int32_t)ch.p);
                ntt_forward<LOGN>(x, tb + team * Sh::TBUF, tt, team, ch);
                const uint4* kp = a.key + ((((size_t)i * L + lvl) * 2 + row) * kChannels + team) * (key_block_words(N) / 4);
#pragma unroll
                for (int rr = 0; rr < 8; ++rr) {
                    const uint4 ka = __ldg(kp + rr * S + tt);
                    const uint4 kb = __ldg(kp + (8 + rr) * S + tt);
                    const uint32_t kav[4] = {ka.x, ka.y, ka.z, ka.w};
                    const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int r = rr * 4 + e;
                        oa[r] = reduce_once(oa[r] + montmul(x[r], kav[e], ch.p, ch.pinv_neg), ch.two_p);
                        ob[r] = reduce_once(ob[r] + montmul(x[r], kbv[e], ch.p, ch.pinv_neg), ch.two_p);
                    }
                }
            }
        }
        ntt_inverse<LOGN>(oa, tb + team * Sh::TBUF, tt, team, ch);
#pragma unroll
        for (int r = 0; r < 32; ++r) xb[(team * 2 + 0) * N + r * S + tt] = reduce_once(oa[r], ch.p);
        ntt_inverse<LOGN>(ob, tb + team * Sh::TBUF, tt, team, ch);
#pragma unroll
        for (int r = 0; r < 32; ++r) xb[(team * 2 + 1) * N + r * S + tt] = reduce_once(ob[r], ch.p);
        __syncthreads();

        // CRT -> applyIntt's centred mod-q value mod 2^T, then accumulateTrlwe (trlwe.h:268-274)
        for (int idx = tid; idx < 2 * N; idx += nth) {
            const int o = idx >= N;
            const int j = idx - o * N;
            const int64_t v = crt_to_torus<T>(xb[(0 * 2 + o) * N + j], xb[(1 * 2 + o) * N + j],
                                              xb[(2 * 2 + o) * N + j], a.crt);
            if constexpr (T == 32) acc[idx] = (int32_t)((uint32_t)acc[idx] + (uint32_t)v);
            else acc[idx] = sext<56>((int64_t)((uint64_t)acc[idx] + (uint64_t)v));
        }
        __syncthreads();
    }

    if (a.acc_out) {
        int64_t* dst = a.acc_out + (size_t)ct * 2 * N;
        for (int idx = tid; idx < 2 * N; idx += nth) dst[idx] = (int64_t)acc[idx];
    }
    if (a.big_out) {
        // extractTlweFromTrlwe(out, acc, 0): a'[j] = j ? -a[N-j] : a[0], b' = b[0], rescaled 2^T -> 2^32
        int32_t* dst = a.big_out + (size_t)ct * (N + 1);
        for (int j = tid; j <= N; j += nth) {
            TorusT x = j == N ? acc[N] : (j == 0 ? acc[0] : tneg<T>(acc[N - j]));
            if constexpr (T == 32) dst[j] = (int32_t)x;
            else dst[j] = (int32_t)modswitch_down((int64_t)x, T - 32, 32);
        }
    }
}

constexpr int kKsTile = 8;      // ciphertexts per block
constexpr int kKsCols = 128;    // output columns per block (= threads)
constexpr int kKsChunk = 32;    // input coefficients per digit refresh
constexpr int kKsMaxT = 16;

__global__ void __launch_bounds__(kKsCols) keyswitch_kernel(const KsArgs a) {
    __shared__ int8_t sdig[kKsTile][kKsChunk][kKsMaxT];
    __shared__ int32_t sb[kKsTile];
    const int x = blockIdx.y * kKsCols + threadIdx.x;
    const int c0 = blockIdx.x * kKsTile;
    const int nb = a.n + 1;
    uint32_t acc[kKsTile];
#pragma unroll
    for (int c = 0; c < kKsTile; ++c) acc[c] = 0;
    if (threadIdx.x < kKsTile) {
        const int ct = c0 + threadIdx.x;
        sb[threadIdx.x] = ct < a.count ? a.big_in[(size_t)ct * (a.kN + 1) + a.kN] : 0;
    }
    for (int i0 = 0; i0 < a.kN; i0 += kKsChunk) {
        __syncthreads();
        for (int e = threadIdx.x; e < kKsTile * kKsChunk; e += kKsCols) {
            const int c = e / kKsChunk, ii = e % kKsChunk;
            const int ct = c0 + c, i = i0 + ii;
            const int32_t v = (ct < a.count && i < a.kN) ? a.big_in[(size_t)ct * (a.kN + 1) + i] : 0;
            zero_mean_digits<uint32_t, 32>((uint32_t)v, a.t, a.ks_radix_bits,
                                           [&](int level, int d) { sdig[c][ii][level] = (int8_t)d; });
        }
        __syncthreads();
        if (x < nb) {
            const int iend = min(kKsChunk, a.kN - i0);
            for (int ii = 0; ii < iend; ++ii) {
                const int32_t* row = a.ksk + ((size_t)(i0 + ii) * a.t) * nb + x;
                for (int j = 0; j < a.t; ++j) {
                    const uint32_t w = (uint32_t)__ldg(row + (size_t)j * nb);
#pragma unroll
                    for (int c = 0; c < kKsTile; ++c) acc[c] += (uint32_t)(int32_t)sdig[c][ii][j] * w;
                }
            }
        }
    }
    if (x < nb) {
#pragma unroll
        for (int c = 0; c < kKsTile; ++c) {
            const int ct = c0 + c;
            if (ct < a.count) a.out[(size_t)ct * nb + x] = (int32_t)((x == a.n ? (uint32_t)sb[c] : 0u) - acc[c]);
        }
    }
}

template <int LOGN, int T>
int launch_br_t(const BrArgs& a, void* stream) {
    const size_t smem = br_smem_bytes(LOGN, T, a.n, a.L);
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(blind_rotate_kernel<LOGN, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
            cudaSuccess)
            return -1;
        attr_set = true;
    }
    blind_rotate_kernel<LOGN, T><<<a.count, 3 * TeamShape<LOGN>::S, smem, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

size_t br_smem_bytes(int logN, int torus_bits, int n, int L) {
    const size_t N = (size_t)1 << logN;
    const size_t tbuf = N + N / 32;
    size_t b = kChannels * tbuf * 4 + kChannels * 2 * N * 4;
    b += 2 * N * (torus_bits == 32 ? 4 : 8);
    b += 2 * (size_t)L * N * 2;
    b += ((size_t)n + 1) * 2;
    return (b + 15) & ~(size_t)15;
}

int launch_keyconv(int logN, const KeyConvArgs& a, void* stream) {
    if (logN == 10) keyconv_kernel<10><<<a.polys, 3 * TeamShape<10>::S, 0, (cudaStream_t)stream>>>(a);
    else if (logN == 11) keyconv_kernel<11><<<a.polys, 3 * TeamShape<11>::S, 0, (cudaStream_t)stream>>>(a);
    else return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_blind_rotate(int logN, int torus_bits, const BrArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    if (logN == 10 && torus_bits == 32) return launch_br_t<10, 32>(a, stream);
    if (logN == 10 && torus_bits == 56) return launch_br_t<10, 56>(a, stream);
    if (logN == 11 && torus_bits == 32) return launch_br_t<11, 32>(a, stream);
    if (logN == 11 && torus_bits == 56) return launch_br_t<11, 56>(a, stream);
    return -1;
}

int launch_keyswitch(const KsArgs& a, void* stream) {
    if (a.count <= 0) return 0;
    if (a.t > kKsMaxT) return -1;
    dim3 grid((a.count + kKsTile - 1) / kKsTile, (a.n + 1 + kKsCols - 1) / kKsCols);
    keyswitch_kernel<<<grid, kKsCols, 0, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yg
