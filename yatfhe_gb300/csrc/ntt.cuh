// ntt.cuh -- negacyclic NTT of one polynomial in one RNS channel by a "team" of N/32
// threads (one warp at N = 1024, two at N = 2048), 32 residues per thread in registers.
//
// Forward transform = Cooley-Tukey with psi^brv(k) twiddles (output in bit-reversed
// slots), inverse = Gentleman-Sande with psi^-brv(k) (bit-reversed in, natural out,
// NOT scaled by N^-1: that factor is folded into the stored key).  For a stage on index
// bit s the twiddle is psi^brv(2^(logN-1-s) + (j >> (s+1))).  The tables keep that index
// for the stages on the top five bits (the first 32 entries, also in __constant__), but
// store the per-thread twiddles of the other stages stage by stage with the thread's
// group index fastest: entry (gid, k) of the stage whose natural entries are
// 2^(9-sp) + gid K + k (K = 2^(4-sp) per thread) sits at 2^(9-sp) + k 32 + gid, and at
// N = 2048 the index-bit-0 stage's entry 1024 + gid 32 + r sits at 1024 + r 32 + gid.  A
// warp's twiddle load then reads one contiguous run of 256 bytes instead of 32 lines.
//
// Layouts (tt = thread index in the team, S = N/32 threads):
//   natural : register r holds coefficient j = r*S + tt           (the 5 top index bits)
//   slot    : N = 1024: register r holds slot j = tt*32 + r        (the 5 low index bits)
//             N = 2048: register r holds slot j = (tt>>1)*64 + 2r + (tt&1); index bit 0 is
//                       split across the lane pair (tt, tt^1) and done with shuffles.
// Forward: natural -> 5 register stages -> transpose through shared memory -> slot -> 5
// register stages (+ the shuffle stage at N = 2048).  Inverse mirrors it.  Pointwise
// products happen in the slot layout, so the key is stored in that layout.
//
// Prime sets 1 and 2 (p < 2^26.48) run every stage on biased values (rns.cuh,
// ct_bfly_b): the forward input carries an offset of at least 2p per stage (fwd_bias_*), so
// no butterfly wraps and none reduces; outputs stay below 46p.  Its inverse at N = 1024 is
// a Cooley-Tukey (decimation-in-time) transform too: on bit-reversed slots with
// omega = psi^2, the stages on slot bits 0..4 take twiddles psi^-((N / 2^sp) m) that depend
// only on the register index (constant bank; bit 0 needs none), the stages on bits 5..9
// per-thread twiddles psi^-((N / 2^(5+sp)) (m 32 + tt)) (entries 32 (2^sp - 1) + m 32 + tt of
// the inverse table), and a final twist by psi^-j (entries 992 + j) turns the cyclic
// inverse into the negacyclic one.  Other shapes keep the Gentleman-Sande inverse with
// psi^-brv(k) twiddles.
#pragma once
#include "rns.cuh"

namespace yg {

__device__ __forceinline__ int tpad(int j) { return j + (j >> 5); }

// words per digit-product table (ntt_forward TAB = 2): digits -64..64 at offset 64
constexpr int kTab0WordsNtt = 132;

// The per-thread twiddle addresses depend only on the thread, so the compiler would hoist
// those loads out of the CMux loop and keep them live in registers across the whole step;
// reading the table pointer through a volatile move inside each transform keeps the loads
// next to their use (measured faster, and it frees registers for the butterflies).
__device__ __forceinline__ const uint2* pinned(const uint2* t) {
    const uint2* r;
    asm volatile("mov.b64 %0, %1;" : "=l"(r) : "l"(t));
    return r;
}

// The first 32 twiddles of each table: every thread of a team uses the same ones in the
// natural-layout stages, so they come from the constant cache.
// [prime set][logN-10][channel][fwd, inv][k]
__constant__ uint2 c_tw_head[kPrimeSets][2][kChannels][2][32];

template <int LOGN>
struct TeamShape {
    static constexpr int N = 1 << LOGN;
    static constexpr int S = N / 32;
    static constexpr int WARPS = S / 32;
    static constexpr int TBUF = N + N / 32;  // words of one transpose buffer
    static_assert(LOGN == 10 || LOGN == 11, "team NTT supports N = 1024 and 2048");
};

// Barrier over the warps of one channel team: a warp barrier at N = 1024, named barrier
// 1 + bar (64 threads) at N = 2048; `bar` is unique per team in the CTA, and id 0 is left to
// __syncthreads.
template <int LOGN>
__device__ __forceinline__ void team_sync(int bar) {
    if constexpr (LOGN == 10) {
        __syncwarp();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(1 + bar), "r"(64) : "memory");
    }
}

// Offset of the forward transform's input.  Prime set 1: 2p per stage on top of the value
// (signed digits |d| < p: one more p), so the biased butterflies never wrap; prime set 0:
// p, which makes signed digits non-negative.
template <int LOGN, int PS>
__device__ __forceinline__ uint32_t fwd_bias_digits(uint32_t p) { return PS != 0 ? (2 * LOGN + 1) * p : p; }
// The same for residues already in [0, p).
template <int LOGN, int PS>
__device__ __forceinline__ uint32_t fwd_bias_residues(uint32_t p) { return PS != 0 ? 2 * LOGN * p : 0; }

template <int LOGN>
__device__ __forceinline__ int slot_pos(int tt, int r) {
    if constexpr (LOGN == 10) return tt * 32 + r;
    else return (tt >> 1) * 64 + 2 * r + (tt & 1);
}

// The slot of register r of thread tt in the forward transform's output (the layout of the
// pointwise products and of the stored key): slot_pos at N = 1024; at N = 2048 each lane of
// a pair holds whole index-bit-0 pairs, the even lane pairs 0..15 and the odd lane pairs
// 16..31, the pair's U slot in register k and its V slot in register 16 + k.
template <int LOGN>
__host__ __device__ __forceinline__ int slot_pos_out(int tt, int r) {
    if constexpr (LOGN == 10) return tt * 32 + r;
    else return (tt >> 1) * 64 + 2 * ((r & 15) + ((tt & 1) << 4)) + (r >> 4);
}

// PS is the prime set (rns.cuh) of `ch`: it picks the constant-bank twiddles and the
// reduction schedule of the forward transform.
// TAB = 1: the input holds signed digits d (|d| <= 64, as int32) instead of residues, and the
// first stage (pairs j, j + N/2, twiddle psi^(N/2)) reads psi^(N/2) d mod p from `tab`
// (indexed by d) instead of multiplying: x' = d_x + p + t, y' = d_x + 3p - t, both < 4p as
// in the residue path.
// TAB = 2 (prime set 1): the first two stages at once from five tables T_w[d] = w d mod p,
// tab[t kTab0Words + d] for w = w1, w2, w1 w2, w3, w1 w3 (w1 = psi^brv(1), the first stage's
// twiddle; w2, w3 = psi^brv(2), psi^brv(3), the second's): for the digits d0..d3 of registers
// r, r + 8, r + 16, r + 24 (r < 8) the two stages give
//   d0 + T1[d2] + T2[d1] + T12[d3],  d0 + T1[d2] - T2[d1] - T12[d3],
//   d0 - T1[d2] + T3[d1] - T13[d3],  d0 - T1[d2] - T3[d1] + T13[d3]
// on a (2 LOGN - 1) p offset (2p for each stage left): five lookups and no multiply for
// four outputs, where the two radix-2 stages take two lookups and two Shoup products.
template <int LOGN, int PS, int TAB = 0>
__device__ __forceinline__ void ntt_forward(uint32_t (&a)[32], uint32_t* tb, int tt, int team, int bar, const Chan& ch,
                                            const uint32_t* tab = nullptr) {
    constexpr int S = TeamShape<LOGN>::S;
    const uint32_t p = ch.p, two_p = ch.two_p;
    const uint32_t neg_p = 0u - p;
    if constexpr (TAB == 2) {
        static_assert(PS == 1, "the two-stage tables are built for prime set 1");
        constexpr int W = kTab0WordsNtt;
        // offset (2 LOGN - 1) p: every output at least (2 LOGN - 4) p - 64, two p per stage left
        const uint32_t boff = (2 * LOGN - 1) * p;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int d0 = (int)a[r], d1 = (int)a[r + 8], d2 = (int)a[r + 16], d3 = (int)a[r + 24];
            const uint32_t t1 = tab[d2], t2 = tab[W + d1], t12 = tab[2 * W + d3];
            const uint32_t t3 = tab[3 * W + d1], t13 = tab[4 * W + d3];
            const uint32_t base = (uint32_t)d0 + boff;
            const uint32_t hi = base + t1, lo = base - t1;
            a[r] = hi + t2 + t12;
            a[r + 8] = hi - t2 - t12;
            a[r + 16] = lo + t3 - t13;
            a[r + 24] = lo - t3 + t13;
        }
    } else if constexpr (TAB == 1) {
        // prime set 1: offset 2p for each of the LOGN - 1 stages left, and p for t < p
        const uint32_t bx = PS != 0 ? 2 * LOGN * p : p, by = PS != 0 ? 2 * LOGN * p : 3 * p;
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const int dx = (int)a[r], dy = (int)a[r + 16];
            const uint32_t t = tab[dy];
            a[r] = (uint32_t)dx + bx + t;
            a[r + 16] = (uint32_t)dx + by - t;
        }
    }
    // Input residues < 2p; every butterfly adds at most 2p to the bound of its x input.
    // Prime set 0 (p < 2^29, 8p < 2^32): natural-layout stages 4p, 6p, 8p, reduce -> 6p, 8p;
    // slot-layout stages reduce -> 6p, 8p, reduce -> 6p, 8p, reduce -> 6p (then the N = 2048
    // shuffle stage, reduce -> 6p).  Output < 8p.  Prime set 1 (p < 2^26.48): biased
    // butterflies, no reduction; the input offset (fwd_bias_*, or the table stage's 2 LOGN p)
    // falls by less than 2p per stage and the value grows by less than 2p, so the output
    // stays below (4 LOGN + 1) p + 2^14 < 46p < 2^32.
#pragma unroll
    for (int sp = TAB == 2 ? 2 : (TAB ? 3 : 4); sp >= 0; --sp) {
        const int h = 1 << sp;
#pragma unroll
        for (int r = 0; r < 32; ++r) {
            if (r & h) continue;
            const uint2 w = c_tw_head[PS][LOGN - 10][team][0][(1 << (4 - sp)) + (r >> (sp + 1))];
            if constexpr (PS != 0) ct_bfly_b(a[r], a[r + h], w, neg_p);
            else ct_bfly(a[r], a[r + h], w, p, two_p, sp == 1);
        }
    }
    team_sync<LOGN>(bar);
#pragma unroll
    for (int r = 0; r < 32; ++r) tb[tpad(r * S + tt)] = a[r];
    team_sync<LOGN>(bar);
#pragma unroll
    for (int r = 0; r < 32; ++r) a[r] = tb[tpad(slot_pos<LOGN>(tt, r))];
    const int gid = LOGN == 10 ? tt : (tt >> 1);
#pragma unroll
    for (int sp = 4; sp >= 0; --sp) {
        const int h = 1 << sp;
        const uint2* tw = pinned(ch.twf) + (1 << (9 - sp)) + gid;
#pragma unroll
        for (int r = 0; r < 32; ++r) {
            if (r & h) continue;
            const uint2 w = __ldg(&tw[(r >> (sp + 1)) * 32]);
            if constexpr (PS != 0) ct_bfly_b(a[r], a[r + h], w, neg_p);
            else ct_bfly(a[r], a[r + h], w, p, two_p, (sp & 1) == 0);
        }
    }
    if constexpr (LOGN == 11) {
        // index bit 0: the pair of register r is (U, V) = (even lane's a[r], odd lane's a[r]).
        // The even lane takes pairs 0..15 and the odd lane pairs 16..31: one exchange of 16
        // values each way, and each lane runs 16 whole butterflies.  Output (the split slot
        // layout, slot_pos_out): a[k] = U' and a[16 + k] = V' of pair k (even lane) or pair
        // 16 + k (odd lane).
        const bool odd = tt & 1;
        const uint2* tw = pinned(ch.twf) + 1024 + gid + (odd ? 16 * 32 : 0);
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const uint32_t recv = __shfl_xor_sync(0xffffffffu, odd ? a[k] : a[16 + k], 1);
            uint32_t u = odd ? recv : a[k];
            uint32_t v = odd ? a[16 + k] : recv;
            const uint2 w = __ldg(&tw[k * 32]);
            if constexpr (PS != 0) ct_bfly_b(u, v, w, neg_p);
            else ct_bfly(u, v, w, p, two_p, true);
            a[k] = u;
            a[16 + k] = v;
        }
    }
}

// Input residues in [0, 2p) in the slot layout; output N times the coefficients in [0, 2p),
// natural layout.
template <int LOGN, int PS>
__device__ __forceinline__ void ntt_inverse(uint32_t (&a)[32], uint32_t* tb, int tt, int team, int bar, const Chan& ch) {
    constexpr int S = TeamShape<LOGN>::S;
    const uint32_t p = ch.p, two_p = ch.two_p;
    if constexpr (PS == 1 && LOGN == 10) {
        const uint32_t neg_p = 0u - p;
        // slot bit 0: twiddle 1, no multiply; offsets 18p / 20p keep the nine biased stages
        // that follow from wrapping: [0, 2p) -> [18p, 22p), at most 40p at the end
        const uint32_t b18 = 18 * p, b20 = 20 * p;
#pragma unroll
        for (int r = 0; r < 32; r += 2) {
            const uint32_t x = a[r], y = a[r + 1];
            a[r] = x + y + b18;
            a[r + 1] = x - y + b20;
        }
#pragma unroll
        for (int sp = 1; sp <= 4; ++sp) {
            const int h = 1 << sp;
#pragma unroll
            for (int r = 0; r < 32; ++r) {
                if (r & h) continue;
                ct_bfly_b(a[r], a[r + h], c_tw_head[PS][0][team][1][h + (r & (h - 1))], neg_p);
            }
        }
        team_sync<LOGN>(bar);
#pragma unroll
        for (int r = 0; r < 32; ++r) tb[tpad(slot_pos<LOGN>(tt, r))] = a[r];
        team_sync<LOGN>(bar);
#pragma unroll
        for (int r = 0; r < 32; ++r) a[r] = tb[tpad(r * S + tt)];
#pragma unroll
        for (int sp = 0; sp <= 4; ++sp) {
            const int h = 1 << sp;
            const uint2* tw = pinned(ch.twi) + 32 * (h - 1) + tt;
#pragma unroll
            for (int r = 0; r < 32; ++r) {
                if (r & h) continue;
                ct_bfly_b(a[r], a[r + h], __ldg(&tw[(r & (h - 1)) * 32]), neg_p);
            }
        }
        // twist by psi^-j, j = r S + tt: the negacyclic transform from the cyclic one
        const uint2* tw = pinned(ch.twi) + 992 + tt;
#pragma unroll
        for (int r = 0; r < 32; ++r) {
            const uint2 w = __ldg(&tw[r * 32]);
            a[r] = mulshoup(a[r], w.x, w.y, p);
        }
        return;
    }
    const int gid = LOGN == 10 ? tt : (tt >> 1);
    if constexpr (LOGN == 11) {
        // index bit 0 on the split slot layout of the forward transform's output: each lane
        // holds whole pairs (a[k], a[16 + k]), runs their 16 butterflies, and one exchange of
        // 16 values each way returns the U outputs to the even lane and the V outputs to the
        // odd lane (register r = pair r) for the stages that follow.
        const bool odd = tt & 1;
        const uint2* tw = pinned(ch.twi) + 1024 + gid + (odd ? 16 * 32 : 0);
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const uint32_t u = a[k], v = a[16 + k];
            const uint2 w = __ldg(&tw[k * 32]);
            const uint32_t su = reduce_once(u + v, two_p);
            const uint32_t dv = mulshoup(u - v + two_p, w.x, w.y, p);
            const uint32_t recv = __shfl_xor_sync(0xffffffffu, odd ? su : dv, 1);
            a[k] = odd ? recv : su;
            a[16 + k] = odd ? dv : recv;
        }
    }
#pragma unroll
    for (int sp = 0; sp <= 4; ++sp) {
        const int h = 1 << sp;
        const uint2* tw = pinned(ch.twi) + (1 << (9 - sp)) + gid;
#pragma unroll
        for (int r = 0; r < 32; ++r) {
            if (r & h) continue;
            gs_bfly(a[r], a[r + h], __ldg(&tw[(r >> (sp + 1)) * 32]), p, two_p);
        }
    }
    team_sync<LOGN>(bar);
#pragma unroll
    for (int r = 0; r < 32; ++r) tb[tpad(slot_pos<LOGN>(tt, r))] = a[r];
    team_sync<LOGN>(bar);
#pragma unroll
    for (int r = 0; r < 32; ++r) a[r] = tb[tpad(r * S + tt)];
#pragma unroll
    for (int sp = 0; sp <= 4; ++sp) {
        const int h = 1 << sp;
#pragma unroll
        for (int r = 0; r < 32; ++r) {
            if (r & h) continue;
            gs_bfly(a[r], a[r + h], c_tw_head[PS][LOGN - 10][team][1][(1 << (4 - sp)) + (r >> (sp + 1))], p, two_p);
        }
    }
}

// ---------------------------------------------------------------- 16-residue inverse
// N = 1024, prime set 1, a team of 64 threads (two warps) with 16 residues per thread: half
// the per-thread chain of the 32-residue inverse, for the latency layout.  Index bits b9..b0
// of a slot or coefficient j, thread tt = (g, beta, gamma) = (tt >> 2, bit 1, bit 0):
//   in     : slot16(tt, q) = g 64 + (8 beta + (q & 7)) 4 + gamma 2 + (q >> 3)
//   middle : register q holds j = g 64 + q 4 + (tt & 3)          (b5..b2 in registers)
//   out    : register q holds j = q 64 + tt                      (b9..b6 in registers)
// Index bits 0 and 1 first (bit 1 across lanes tt ^ 1: each lane sends 8 values, receives 8
// and runs 8 whole butterflies), 2..4 in registers, bit 5 across lanes tt ^ 2, a transpose,
// bits 6..9 in registers and the psi^-j twist.  Twiddles from a plain table inv16[e] =
// psi^-e (with Shoup companions) in natural order.  Same biased arithmetic as the
// 32-residue inverse (rns.cuh: ct_bfly_b).

__device__ __forceinline__ int slot16(int tt, int q) {
    return (tt >> 2) * 64 + (8 * ((tt >> 1) & 1) + (q & 7)) * 4 + (tt & 1) * 2 + (q >> 3);
}

// barrier over the 64 threads of a 16-residue team: named barrier 1 + bar
__device__ __forceinline__ void team16_sync(int bar) { asm volatile("bar.sync %0, 64;" ::"r"(1 + bar) : "memory"); }

// Input residues in [0, 2p) at slot16; output N times the coefficients in [0, 2p), natural.
__device__ __forceinline__ void ntt16_inverse(uint32_t (&a)[16], uint32_t* tb, int tt, int bar, const Chan& ch,
                                              const uint2* inv16) {
    const uint32_t p = ch.p, neg_p = 0u - p;
    const int g = tt >> 2, gamma = tt & 1;
    const uint2* tw = pinned(inv16);
    // index bit 0 (registers k, 8 + k): twiddle 1; offsets 18p / 20p as in the 32-residue inverse
    {
        const uint32_t b18 = 18 * p, b20 = 20 * p;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t x = a[k], y = a[8 + k];
            a[k] = x + y + b18;
            a[8 + k] = x - y + b20;
        }
    }
    // index bit 1 (lanes tt, tt ^ 1): gamma = 0 takes the pairs with bit 0 clear (twiddle 1),
    // gamma = 1 those with bit 0 set (psi^-512)
    {
        const uint2 w = __ldg(&tw[gamma ? 512 : 0]);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t recv = __shfl_xor_sync(0xffffffffu, gamma ? a[k] : a[8 + k], 1);
            uint32_t u = gamma ? recv : a[k];
            uint32_t v = gamma ? a[8 + k] : recv;
            ct_bfly_b(u, v, w, neg_p);
            a[k] = u;
            a[8 + k] = v;
        }
    }
    // index bits 2, 3, 4: registers within each half (half = index bit 1)
#pragma unroll
    for (int s = 2; s <= 4; ++s) {
        const int hk = 1 << (s - 2);
#pragma unroll
        for (int half = 0; half < 2; ++half)
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (k & hk) continue;
                const int jmod = (k & (hk - 1)) * 4 + 2 * half + gamma;
                ct_bfly_b(a[half * 8 + k], a[half * 8 + k + hk], __ldg(&tw[(1024 >> s) * jmod]), neg_p);
            }
    }
    // index bit 5 (lanes tt, tt ^ 2): beta = 0 takes the pairs with bit 1 clear
    {
        const bool hi = (tt >> 1) & 1;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t recv = __shfl_xor_sync(0xffffffffu, hi ? a[k] : a[8 + k], 2);
            uint32_t u = hi ? recv : a[k];
            uint32_t v = hi ? a[8 + k] : recv;
            ct_bfly_b(u, v, __ldg(&tw[32 * (k * 4 + (hi ? 2 : 0) + gamma)]), neg_p);
            a[k] = u;
            a[8 + k] = v;
        }
    }
    team16_sync(bar);
#pragma unroll
    for (int q = 0; q < 16; ++q) tb[tpad(g * 64 + q * 4 + (tt & 3))] = a[q];
    team16_sync(bar);
#pragma unroll
    for (int q = 0; q < 16; ++q) a[q] = tb[tpad(q * 64 + tt)];
    // index bits 6..9 (registers, natural layout)
#pragma unroll
    for (int sp = 0; sp <= 3; ++sp) {
        const int h = 1 << sp;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            if (q & h) continue;
            ct_bfly_b(a[q], a[q + h], __ldg(&tw[(1024 >> (6 + sp)) * ((q & (h - 1)) * 64 + tt)]), neg_p);
        }
    }
    // twist by psi^-j, j = q 64 + tt
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const uint2 w = __ldg(&tw[q * 64 + tt]);
        a[q] = mulshoup(a[q], w.x, w.y, p);
    }
}

}  // namespace yg
