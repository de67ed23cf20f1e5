// crt_kernels.cu -- the approximate-CRT blind rotation (blindRotateApproxCRTNtt,
// yatfhe/src/blind_rotate.cpp:577-589) on the GPU.
//
// The reference's CRT variant works on the torus Q_CRT = 251 241 239 233: the accumulator is
// kept as d = 4 residue samples (int8, centred mod q_d; the two low primes scaled by taoU), and
// each CMux step (controlMuxApproxCRTNtt, yatfhe/src/cmux.cpp:45-57) rotates every residue
// sample, decomposes the rotated difference into two "high" digits by the approximate CRT
// gadget (decompTrlweApproxCrt / broadcastTrlweApproxCrt, yatfhe/src/crt.cpp:102-164),
// multiplies the digits with the key's residue rows in NttNative24's field (the 24-bit prime
// 2^24 - 2^14 + 1, yatfhe/src/ntt24.cpp) and brings each product back to a centred residue
// mod q_d (applyIntt, ntt24.cpp:222-240) before the accumulation mod q_d.  What matters for
// bit-exactness is the integer X mod (2^24 - 2^14 + 1) of each negacyclic product sum, which
// any exact transform gives; here the team NTT of the main blind rotation (ntt.cuh) runs on
// prime set 2, which is that prime.
//
// One CTA per ciphertext, one team (N/32 threads) per residue prime d: per step all threads
// rotate and decompose (one pass over the 2N coefficients, reading all four residue samples),
// then team d transforms its four digit polynomials (2 levels x 2 rows), accumulates the
// Montgomery products with the key rows of prime d for both outputs, runs the two inverse
// transforms and updates its own residue sample; a CTA barrier closes the step.
#include <cuda_runtime.h>

#include <cstdint>

#include "ntt.cuh"
#include "pbs_kernels.cuh"

namespace yg {

namespace {

constexpr int kCrtPS = 2;  // prime set of 2^24 - 2^14 + 1 (rns.cuh)

// the four residue primes (QD_CRT, yatfhe/include/yatfhe/torus.h:45): two high, two low
__host__ __device__ constexpr int crt_q(int d) { return d == 0 ? 251 : d == 1 ? 241 : d == 2 ? 239 : 233; }

// The centred residue in [-(q-1)/2, (q-1)/2] of |x| < 1.5 q (intModP, numeric.cpp:104-112).
__device__ __forceinline__ int cmod_near(int x, int q) {
    const int h = (q - 1) >> 1;
    return x > h ? x - q : (x < -h ? x + q : x);
}

// The centred residue of any |x| < 2^24 mod an odd q in (2^7, 2^8): x + 2^24 rounded up to a
// multiple of q is non-negative and below 2^25, and floor(u m / 2^39) with m = ceil(2^39 / q)
// (below 2^32) is floor(u / q) exactly there (u m / 2^39 exceeds u / q by less than 2^-14, and
// frac(u / q) <= 1 - 1/q).
__device__ __forceinline__ int cmod_any(int x, int q, uint32_t m) {
    const uint32_t off = (uint32_t)(((1u << 24) / q + 1) * q);
    const uint32_t u = (uint32_t)(x + (int)off);
    const uint32_t qq = (uint32_t)(((uint64_t)u * m) >> 39);
    const int r = (int)(u - qq * (uint32_t)q);
    return r > ((q - 1) >> 1) ? r - q : r;
}

__device__ __forceinline__ uint32_t crt_magic(int q) { return (uint32_t)(((1ull << 39) + q - 1) / q); }

// The key rows of one (i, d, level, row): each of the two key polynomials (the row's output
// a, then b) into the slot layout of the forward transform, times N^-1 2^32 (the inverse
// transform's scale and the Montgomery factor of the MAC), reduced, in the interleaved
// layout the MAC reads as uint4.
template <int LOGN>
__global__ void __launch_bounds__(2 * TeamShape<LOGN>::S) crt_keyconv_kernel(const CrtKeyConvArgs a) {
    using Sh = TeamShape<LOGN>;
    constexpr int N = Sh::N, S = Sh::S;
    __shared__ uint32_t tb[2 * Sh::TBUF];
    const int blk = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = warp / Sh::WARPS;
    const int tt = (warp % Sh::WARPS) * 32 + lane;
    const Chan ch = a.ch;
    const int8_t* src = a.bsk8 + ((size_t)blk * 2 + c) * N;
    uint32_t x[32];
    const uint32_t bias = fwd_bias_residues<LOGN, kCrtPS>(ch.p);
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        const int v = src[r * S + tt];
        x[r] = (uint32_t)(v < 0 ? v + (int)ch.p : v) + bias;
    }
    ntt_forward<LOGN, kCrtPS>(x, tb + c * Sh::TBUF, tt, 0, c, ch);
    uint32_t* dst = a.key + (size_t)blk * key_block_words(N);
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        const uint32_t y = reduce_once(reduce_once(mulshoup(x[r], a.scale, a.scale_s, ch.p), ch.two_p), ch.p);
        dst[((c * 8 + (r >> 2)) * S + tt) * 4 + (r & 3)] = y;
    }
}

// Two CTAs per SM (a register cap of 128 at N = 2048): measured 10.1 k against 7.4 k rotations/s
// with one CTA of 211 registers (n = 680, N = 2048, 1,216 ciphertexts, outputs identical).
template <int LOGN>
__global__ void __launch_bounds__(kCrtD * TeamShape<LOGN>::S, 2) crt_blind_rotate_kernel(const CrtBrArgs a) {
    using Sh = TeamShape<LOGN>;
    constexpr int N = Sh::N, S = Sh::S, T = kCrtD * S;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* xb = reinterpret_cast<uint32_t*>(smem);                 // [d][TBUF] transposes
    int8_t* acc = reinterpret_cast<int8_t*>(xb + kCrtD * Sh::TBUF);  // [d][2][N] residue samples
    int8_t* hi = acc + kCrtD * 2 * N;                                 // [level][row][N] digits
    int16_t* ra = reinterpret_cast<int16_t*>(hi + kCrtDh * 2 * N);    // [n] rotations mod 2N

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int d = warp / Sh::WARPS;                     // this team's residue prime
    const int tt = (warp % Sh::WARPS) * 32 + lane;
    const int q = crt_q(d);
    const uint32_t magic = crt_magic(q);
    const Chan ch = a.ch;
    const uint32_t pinv = 0u - ch.pinv_neg;
    uint32_t* mine = xb + d * Sh::TBUF;
    const int n = a.n;

    for (int ct = blockIdx.x; ct < a.count; ct += gridDim.x) {
        // decompTrlweMcrt (yatfhe/include/yatfhe/trlwe.h:333-371): longModP(taoU_d v, q_d)
        const int32_t* in = a.acc_in + (size_t)ct * 2 * N;
        for (int idx = tid; idx < 2 * N; idx += T) {
            const int64_t v = in[idx];
#pragma unroll
            for (int dd = 0; dd < kCrtD; ++dd) {
                const int64_t qd = crt_q(dd);
                int64_t r = (v * a.tao_u[dd]) % qd;
                r = r > (qd - 1) / 2 ? r - qd : (r < -((qd - 1) / 2) ? r + qd : r);
                acc[dd * 2 * N + idx] = (int8_t)r;
            }
        }
        const int32_t* rot = a.rot + (size_t)ct * n;
        for (int i = tid; i < n; i += T) {
            int r = rot[i] % (2 * N);
            ra[i] = (int16_t)(r < 0 ? r + 2 * N : r);
        }
        __syncthreads();

        for (int i = 0; i < n; ++i) {
            const int t2 = ra[i];
            if (t2 == 0) continue;  // the reference skips a_i = 0; a multiple of 2N rotates by nothing
            const bool wrap = t2 >= N;
            const int at = wrap ? t2 - N : t2;
            // rotateInt8PolynomialMinusOne per residue sample, then decompTrlweApproxCrt:
            // low = (qLow / 239) tmp_2 + (qLow / 233) tmp_3, digit_l = intModP(tmp_l - low, q_l)
            for (int idx = tid; idx < 2 * N; idx += T) {
                const int r = idx >= N;
                const int j = idx - r * N;
                int tmp[kCrtD];
#pragma unroll
                for (int dd = 0; dd < kCrtD; ++dd) {
                    const int8_t* A = acc + (dd * 2 + r) * N;
                    int v = j < at ? -(int)A[j - at + N] : (int)A[j - at];
                    if (wrap) v = -v;
                    tmp[dd] = cmod_near(v - (int)A[j], crt_q(dd));
                }
                const int low = 233 * tmp[2] + 239 * tmp[3];
#pragma unroll
                for (int l = 0; l < kCrtDh; ++l) {
                    const int ql = crt_q(l);
                    int v = (tmp[l] - low) % ql;
                    v = v > (ql - 1) / 2 ? v - ql : (v < -((ql - 1) / 2) ? v + ql : v);
                    hi[(l * 2 + r) * N + j] = (int8_t)v;
                }
            }
            __syncthreads();

            // externalProductTrgswApproxCrtNtt (yatfhe/src/trgsw.cpp:607-657) for prime d:
            // the digits broadcast to q_d (broadcastTrlweApproxCrt), forward transforms, products
            // with the key rows summed for both outputs (Montgomery terms in (-p, p) on a 4p bias)
            uint32_t oa[32], ob[32];
#pragma unroll
            for (int r = 0; r < 32; ++r) oa[r] = ob[r] = 4 * ch.p;
            const int qh = q >> 1;
#pragma unroll 1
            for (int lr = 0; lr < kCrtDh * 2; ++lr) {
                const int8_t* dg = hi + lr * N;
                uint32_t x[32];
                const uint32_t bias = fwd_bias_digits<LOGN, kCrtPS>(ch.p);
#pragma unroll
                for (int r = 0; r < 32; ++r) {
                    int v = dg[r * S + tt];
                    if (v > qh || v < -qh) v = cmod_near(v, q);
                    x[r] = (uint32_t)v + bias;
                }
                ntt_forward<LOGN, kCrtPS>(x, mine, tt, 0, d, ch);
                const uint4* kp = reinterpret_cast<const uint4*>(
                    a.key + ((((size_t)i * kCrtD + d) * kCrtDh * 2) + lr) * key_block_words(N));
#pragma unroll
                for (int rr = 0; rr < 8; ++rr) {
                    const uint4 ka = __ldg(kp + rr * S + tt);
                    const uint4 kb = __ldg(kp + (8 + rr) * S + tt);
                    const uint32_t kav[4] = {ka.x, ka.y, ka.z, ka.w};
                    const uint32_t kbv[4] = {kb.x, kb.y, kb.z, kb.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int r = rr * 4 + e;
                        oa[r] += montdiff<true>(x[r], kav[e], ch.p, pinv);
                        ob[r] += montdiff<true>(x[r], kbv[e], ch.p, pinv);
                    }
                }
            }
            // inverse transforms; X mod p centred (HALF_MOD), then centred mod q_d (applyIntt),
            // then accumulateTrlweModP: acc_d = longModP(res + acc_d, q_d)
            const int32_t half = (int32_t)((ch.p + 1) >> 1);
#pragma unroll 1
            for (int c = 0; c < 2; ++c) {
                if (c == 1) {
#pragma unroll
                    for (int r = 0; r < 32; ++r) oa[r] = ob[r];
                }
#pragma unroll
                for (int r = 0; r < 32; ++r) oa[r] = reduce_once(reduce_once(oa[r], 2 * ch.two_p), ch.two_p);
                ntt_inverse<LOGN, kCrtPS>(oa, mine, tt, 0, d, ch);
                int8_t* A = acc + (d * 2 + c) * N;
#pragma unroll
                for (int r = 0; r < 32; ++r) {
                    const uint32_t y = reduce_once(oa[r], ch.p);
                    const int centred = (int32_t)y >= half ? (int)y - (int)ch.p : (int)y;
                    const int res = cmod_any(centred, q, magic);
                    const int j = r * S + tt;
                    A[j] = (int8_t)cmod_near(res + (int)A[j], q);
                }
            }
            __syncthreads();
        }

        // trlweMcrtToCrt (low primes times taoUInv) and recompTrlweCrt (sum of z_d x_d mod Q)
        int32_t* out = a.acc_out + (size_t)ct * 2 * N;
        for (int idx = tid; idx < 2 * N; idx += T) {
            int64_t s = 0;
#pragma unroll
            for (int dd = 0; dd < kCrtD; ++dd) {
                int64_t v = acc[dd * 2 * N + idx];
                if (dd >= kCrtDh) {
                    const int64_t qd = crt_q(dd);
                    v = (a.tao_u_inv[dd] * v) % qd;
                    v = v > (qd - 1) / 2 ? v - qd : (v < -((qd - 1) / 2) ? v + qd : v);
                }
                s += v * a.z[dd];
            }
            const int64_t Q = a.q_crt;
            int64_t r = s % Q;
            r = r > (Q - 1) / 2 ? r - Q : (r < -(Q / 2) ? r + Q : r);
            out[idx] = (int32_t)r;
        }
        __syncthreads();  // the next ciphertext rewrites the residue samples
    }
}

}  // namespace

size_t crt_br_smem_bytes(int N, int n) {
    const size_t tbuf = (size_t)N + N / 32;
    return kCrtD * tbuf * 4 + (size_t)kCrtD * 2 * N + (size_t)kCrtDh * 2 * N + (size_t)n * 2;
}

int set_crt_twiddle_heads(int logN, const uint2* heads) {
    if (logN != 10 && logN != 11) return -1;
    const size_t per = sizeof(uint2) * kChannels * 2 * 32;
    return cudaMemcpyToSymbol(c_tw_head, heads, per, per * (kCrtPS * 2 + logN - 10)) == cudaSuccess ? 0 : -1;
}

int launch_crt_keyconv(int logN, const CrtKeyConvArgs& a, void* stream) {
    if (a.rows <= 0) return 0;
    if (logN == 10)
        crt_keyconv_kernel<10><<<a.rows, 2 * TeamShape<10>::S, 0, (cudaStream_t)stream>>>(a);
    else if (logN == 11)
        crt_keyconv_kernel<11><<<a.rows, 2 * TeamShape<11>::S, 0, (cudaStream_t)stream>>>(a);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_crt_blind_rotate(int logN, const CrtBrArgs& a, int grid, void* stream) {
    if (a.count <= 0) return 0;
    const size_t smem = crt_br_smem_bytes(1 << logN, a.n);
    auto go = [&](auto kern, int threads) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
        kern<<<grid, threads, smem, (cudaStream_t)stream>>>(a);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    };
    if (logN == 10) return go(crt_blind_rotate_kernel<10>, kCrtD * TeamShape<10>::S);
    if (logN == 11) return go(crt_blind_rotate_kernel<11>, kCrtD * TeamShape<11>::S);
    return -1;
}

int crt_blind_rotate_ctas_per_sm(int logN, int n, int* out) {
    const size_t smem = crt_br_smem_bytes(1 << logN, n);
    auto q = [&](auto kern, int threads) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return -1;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kern, threads, smem) == cudaSuccess ? 0 : -1;
    };
    if (logN == 10) return q(crt_blind_rotate_kernel<10>, kCrtD * TeamShape<10>::S);
    if (logN == 11) return q(crt_blind_rotate_kernel<11>, kCrtD * TeamShape<11>::S);
    return -1;
}

}  // namespace yg
