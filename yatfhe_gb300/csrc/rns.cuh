// rns.cuh -- 32-bit residue arithmetic for the three-prime RNS the GPU bootstrap works in.
//
// The reference multiplies in the NTT domain modulo one 49-bit (TORUS32) or 61-bit
// (TORUS56) prime q (yatfhe/include/yatfhe/torus.h:151,157, ntt_hexl.cpp:183-190).
// What reaches the accumulator is only centred(INTT(sum NTT(d) . K) mod q) mod 2^T
// (yatfhe/src/ntt_hexl.cpp:153-175), i.e. the exact integer X = sum_j d_j * k_j
// (negacyclic, k_j = INTT(K_j) centred) reduced mod q.  |X| < 2^83 for every supported
// parameter set, so the GPU computes X exactly in an RNS of three primes p_c < 2^29
// (product ~2^87) on the 32-bit integer pipes and reduces it mod q once per coefficient.
#pragma once
#include <cstdint>

namespace yg {

constexpr int kChannels = 3;
// Two sets of three primes p == 1 mod 2^13 (negacyclic NTTs up to N = 4096), each the
// largest below its bound, so p2 < p1 < p0 < 2 p2 in both.
//   set 0: below 2^29, product ~2^87, for the 56-bit torus (|X| < 2^82.8 keeps 3.2 bits of
//          margin below M/2); residues up to 8p fit 32 bits, so the forward NTT reduces
//          every other stage;
//   set 1: below 93.37 M (2^26.48), product ~2^79.4, for the 32-bit torus (|X| < 2^71 for
//          every accepted parameter set, 2^66.6 at n=630/N=1024); residues up to 46p fit
//          32 bits, so both transforms run on biased values without any reduction (ntt.cuh:
//          an input offset by 2p per remaining stage keeps x - r >= 0, and 11 stages of
//          growth by < 2p stay below 46p).
//   set 2: the single 24-bit prime 2^24 - 2^14 + 1 (NttNative24's modulus) in every channel
//          slot, for the approximate-CRT blind rotation, whose products are taken mod that
//          prime itself; biased transforms as in set 1.
constexpr int kPrimeSets = 3;
constexpr uint32_t kMod24 = (1u << 24) - (1u << 14) + 1;
constexpr uint32_t kPrimeSet[kPrimeSets][kChannels] = {{536813569u, 536690689u, 536641537u},
                                                       {93356033u, 93290497u, 93192193u},
                                                       {kMod24, kMod24, kMod24}};
__host__ __device__ constexpr int prime_set_for(int torus_bits) { return torus_bits == 32 ? 1 : 0; }

// Per-channel constants the kernels read.
struct Chan {
    uint32_t p;
    uint32_t two_p;
    uint32_t pinv_neg;      // -p^-1 mod 2^32 (Montgomery)
    uint32_t pad;
    const uint2* twf;       // forward twiddles (w, floor(w 2^32 / p)), psi^brv(k), k in [0, N)
    const uint2* twi;       // inverse table (ntt.cuh; 2N entries)
};

// Constants of the CRT recombination and of the reduction mod q (see crt_to_torus).
struct Crt {
    uint32_t p0, p1, p2;
    uint32_t inv_p0_m1, inv_p0_m1_s;     // p0^-1 mod p1, Shoup companion
    uint32_t p0_m2, p0_m2_s;             // p0 mod p2, Shoup companion
    uint32_t inv_p01_m2, inv_p01_m2_s;   // (p0 p1)^-1 mod p2, Shoup companion
    uint32_t half_p2;                    // (p2 - 1) / 2
    uint64_t p01;                        // p0 p1
    uint64_t q;                          // qNtt of the reference
    uint64_t half_q;                     // (q - 1) / 2
    int64_t a2;                          // round(p0 p1 2^32 / q)
    uint32_t a1;                         // round(p0 2^32 / q)
};

#ifdef __CUDACC__
// x * w mod p in [0, 2p) for any 32-bit x, with wp = floor(w 2^32 / p), w < p.
__device__ __forceinline__ uint32_t mulshoup(uint32_t x, uint32_t w, uint32_t wp, uint32_t p) {
    const uint32_t qh = __umulhi(x, wp);
    return x * w - qh * p;
}

// hi(a b) - hi(m p) with m = (a b mod 2^32) p^-1 mod 2^32: the low words of a b and m p are
// equal, so this is exactly (a b - m p) / 2^32 = a b 2^-32 mod p, as a signed value in (-p, p)
// whenever a b < 2^32 p (b < p and any 32-bit a): a
// Montgomery product without the carry fix-up.
// WIDE selects how a b is formed: one 32 x 32 -> 64 multiply, or separate low and high
// halves; the results are identical, the instruction schedules differ (the wide form
// measured faster in the 32-bit-torus kernels, the split form in the 56-bit ones).
template <bool WIDE>
__device__ __forceinline__ uint32_t montdiff(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
    if constexpr (WIDE) {
        const uint64_t ab = (uint64_t)a * b;
        return (uint32_t)(ab >> 32) - __umulhi((uint32_t)ab * pinv, p);
    } else {
        const uint32_t lo = a * b;
        return __umulhi(a, b) - __umulhi(lo * pinv, p);
    }
}

__device__ __forceinline__ uint32_t reduce_once(uint32_t x, uint32_t m) { return min(x, x - m); }

// Forward Cooley-Tukey butterfly, lazy: with x < B the outputs are < B + 2p (y may be any
// 32-bit value).  RED first brings x < 8p down below 4p, so with p < 2^29 a stage may skip
// the reduction whenever its x inputs are known to be below 6p.  (`red` is a constant at
// every call site once the stage loops are unrolled.)
__device__ __forceinline__ void ct_bfly(uint32_t& x, uint32_t& y, uint2 w, uint32_t p, uint32_t two_p, bool red) {
    const uint32_t xr = red ? reduce_once(x, 2 * two_p) : x;
    const uint32_t t = mulshoup(y, w.x, w.y, p);
    x = xr + t;
    y = xr - t + two_p;
}

// Biased Cooley-Tukey butterfly (prime set 1): with r = w y mod p in [0, 2p) (Shoup),
// x' = x + r and y' = x - r, the latter as 2x - x' (no constant operand); the caller keeps
// x >= 2p so y' does not wrap.  Any offset of x and y that is a multiple of p is carried
// along unchanged modulo p.
__device__ __forceinline__ void ct_bfly_b(uint32_t& x, uint32_t& y, uint2 w, uint32_t neg_p) {
    const uint32_t qh = __umulhi(y, w.y);
    const uint32_t xn = x + y * w.x + qh * neg_p;
    y = x + x - xn;
    x = xn;
}

// Inverse Gentleman-Sande butterfly: x, y in [0, 2p) -> [0, 2p).
__device__ __forceinline__ void gs_bfly(uint32_t& x, uint32_t& y, uint2 w, uint32_t p, uint32_t two_p) {
    const uint32_t s = x + y;
    const uint32_t d = x - y + two_p;
    x = reduce_once(s, two_p);
    y = mulshoup(d, w.x, w.y, p);
}

// sign-extend the low `bits` bits of x (the reference's longModPow2, numeric.h:69-71).
template <int BITS>
__device__ __forceinline__ int64_t sext(int64_t x) {
    return (int64_t)((uint64_t)x << (64 - BITS)) >> (64 - BITS);
}

// Residues x_c in [0, p_c) of the exact integer X with |X| < p0 p1 p2 / 2 -> the torus value
// centred(X mod q) mod 2^T, i.e. what applyIntt (yatfhe/src/ntt_hexl.cpp:153-175) returns.
// Garner's mixed radix gives X = v0 + v1 p0 + v2 p0 p1 exactly, the top digit centred; a
// fixed-point estimate of X / q picks the quotient to within one and exact 64-bit arithmetic
// on X mod 2^64 settles it.
template <int T>
__device__ __forceinline__ int64_t crt_to_torus(uint32_t x0, uint32_t x1, uint32_t x2, const Crt& k) {
    // p2 < p1 < p0 < 2 p2 < 2^29: x0 < 2 p1 and x0 < 2 p2 need no reduction before the
    // subtractions, and every intermediate stays below 5 p2 < 2^32
    const uint32_t v1 = reduce_once(mulshoup(x1 + 2 * k.p1 - x0, k.inv_p0_m1, k.inv_p0_m1_s, k.p1), k.p1);
    const uint32_t ms = mulshoup(v1, k.p0_m2, k.p0_m2_s, k.p2);  // v1 p0 mod p2, in [0, 2 p2)
    const uint32_t v2 = reduce_once(mulshoup(x2 + 4 * k.p2 - x0 - ms, k.inv_p01_m2, k.inv_p01_m2_s, k.p2), k.p2);
    const int32_t v2s = v2 > k.half_p2 ? (int32_t)(v2 - k.p2) : (int32_t)v2;
    // X / q = (v2s p0 p1 + v1 p0 + x0) / q ~ (v2s a2 + v1 a1) / 2^32, rounded: the rounding of
    // a2 and a1 (at most 1/2 each) moves it by |v2s| / 2^33 + v1 / 2^33 < 2^-3 and x0 / q is
    // below 2^-19, so |X / q - test| < 0.65 for every |X| < M / 2 (|v2s a2| < 2^61.5 at
    // T = 32, 2^57.3 at T = 56)
    const int64_t num = (int64_t)v2s * k.a2 + (int64_t)((uint64_t)v1 * k.a1);
    const int64_t test = (num + ((int64_t)1 << 31)) >> 32;
    const uint64_t xlo = (uint64_t)x0 + (uint64_t)v1 * k.p0 + (uint64_t)(int64_t)v2s * k.p01;
    int64_t y = (int64_t)(xlo - (uint64_t)test * k.q);
    const int64_t hq = (int64_t)k.half_q, q = (int64_t)k.q;
    // |y| < 0.65 q: one fix-up pass lands in the centred range
    y = y > hq ? y - q : y;
    y = y < -hq ? y + q : y;
    return sext<T>(y);
}
#endif  // __CUDACC__

}  // namespace yg
