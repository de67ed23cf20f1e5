/*
 * ntt_q.h -- exact negacyclic NTT modulo a single prime q < 2^62, header-only C.
 *
 * TEST INFRASTRUCTURE ONLY.  This file belongs to the oracle: it is included by
 * the HEXL-API stand-in (oracle/shim/hexl/hexl.hpp) that the reference sources are
 * compiled against, and by the plain-C restatement of the bootstrap path
 * (oracle/pbs_oracle.c).  Nothing in the shipped library includes it.
 *
 * Convention (the one the reference's NTT-domain key files are written in, as far as
 * the reference pins it -- see yatfhe/include/yatfhe/ntt_hexl.h:34-44 and
 * yatfhe/src/ntt_hexl.cpp:153-175, whose callers need only that
 * INTT(NTT(x) (.) NTT(y)) is the negacyclic product mod q):
 *   psi       = the minimal primitive 2N-th root of unity mod q (smallest integer g in
 *               [2, q) with g^N == -1 mod q), the root HEXL reports through
 *               NTT::GetMinimalRootOfUnity();
 *   forward   : out[i] = sum_j in[j] * psi^((2*brv(i)+1)*j) mod q, i.e. the Cooley-Tukey
 *               "merged" negacyclic transform (Longa-Naehrig 2016, Alg. 1) whose output
 *               lands in bit-reversed order;
 *   inverse   : the Gentleman-Sande transform with psi^-1 that takes that bit-reversed
 *               order back to natural order and multiplies by N^-1 (Alg. 2).
 * Twiddles are kept with Shoup companions (w' = floor(w 2^64 / q)).
 */
#ifndef YATFHE_ORACLE_NTT_Q_H
#define YATFHE_ORACLE_NTT_Q_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 nq_u128;

static inline uint64_t nq_mulmod_slow(uint64_t a, uint64_t b, uint64_t q) {
    return (uint64_t)(((nq_u128)a * b) % q);
}

static inline uint64_t nq_powmod(uint64_t base, uint64_t e, uint64_t q) {
    uint64_t r = 1 % q;
    base %= q;
    while (e) {
        if (e & 1) r = nq_mulmod_slow(r, base, q);
        base = nq_mulmod_slow(base, base, q);
        e >>= 1;
    }
    return r;
}

/* a^-1 mod q for prime q (Fermat). */
static inline uint64_t nq_invmod(uint64_t a, uint64_t q) { return nq_powmod(a, q - 2, q); }

static inline uint64_t nq_shoup_precomp(uint64_t w, uint64_t q) {
    return (uint64_t)(((nq_u128)w << 64) / q);
}

/* x * w mod q with w' = floor(w 2^64 / q); x < 2^64, q < 2^63; result in [0, q). */
static inline uint64_t nq_mulshoup(uint64_t x, uint64_t w, uint64_t wp, uint64_t q) {
    uint64_t qh = (uint64_t)(((nq_u128)x * wp) >> 64);
    uint64_t r = x * w - qh * q;
    return r >= q ? r - q : r;
}

/* Barrett constants for products of two residues: p < q^2 < 2^124. */
typedef struct {
    uint64_t q;
    int s;          /* bit length of q */
    nq_u128 mu;     /* floor(2^(2s) / q) */
} nq_barrett;

static inline nq_barrett nq_barrett_make(uint64_t q) {
    nq_barrett b;
    b.q = q;
    b.s = 64 - __builtin_clzll(q);
    b.mu = (((nq_u128)1) << (2 * b.s)) / q;
    return b;
}

/* a * b mod q for a, b in [0, q). */
static inline uint64_t nq_mulmod(const nq_barrett* br, uint64_t a, uint64_t b) {
    nq_u128 p = (nq_u128)a * b;
    nq_u128 qh = ((p >> (br->s - 1)) * br->mu) >> (br->s + 1);
    uint64_t r = (uint64_t)(p - qh * br->q);
    while (r >= br->q) r -= br->q;
    return r;
}

static inline uint32_t nq_bitrev(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; i++) { r = (r << 1) | (x & 1); x >>= 1; }
    return r;
}

/* Smallest g in [2, q) with g^N == q - 1 (a primitive 2N-th root for power-of-two N). */
static inline uint64_t nq_minimal_root(uint32_t N, uint64_t q) {
    const uint64_t twoN = 2 * (uint64_t)N;
    if ((q - 1) % twoN != 0) return 0;
    /* find one primitive 2N-th root psi0, then the minimum over its odd powers */
    uint64_t psi0 = 0;
    for (uint64_t x = 2; x < q && !psi0; x++) {
        uint64_t c = nq_powmod(x, (q - 1) / twoN, q);
        if (nq_powmod(c, N, q) == q - 1) psi0 = c;
    }
    if (!psi0) return 0;
    uint64_t best = psi0, sq = nq_mulmod_slow(psi0, psi0, q), cur = psi0;
    for (uint64_t k = 1; k < N; k++) {
        cur = nq_mulmod_slow(cur, sq, q); /* psi0^(2k+1) */
        if (cur < best) best = cur;
    }
    return best;
}

typedef struct {
    uint32_t N;
    int logN;
    uint64_t q;
    uint64_t psi;
    uint64_t* w;    /* w[k]  = psi^brv(k),  k in [0, N) */
    uint64_t* wp;
    uint64_t* wi;   /* wi[k] = psi^-brv(k) */
    uint64_t* wip;
    uint64_t ninv, ninvp;
    nq_barrett br;
} nq_plan;

/* Returns 0 on success, -1 if q has no 2N-th root or allocation fails. */
static inline int nq_plan_init(nq_plan* p, uint32_t N, uint64_t q) {
    memset(p, 0, sizeof(*p));
    p->N = N;
    p->logN = 0;
    while ((1u << p->logN) < N) p->logN++;
    p->q = q;
    p->psi = nq_minimal_root(N, q);
    if (!p->psi) return -1;
    p->w = (uint64_t*)malloc(4 * sizeof(uint64_t) * N);
    if (!p->w) return -1;
    p->wp = p->w + N;
    p->wi = p->wp + N;
    p->wip = p->wi + N;
    uint64_t psiinv = nq_invmod(p->psi, q);
    for (uint32_t k = 0; k < N; k++) {
        uint32_t e = nq_bitrev(k, p->logN);
        p->w[k] = nq_powmod(p->psi, e, q);
        p->wp[k] = nq_shoup_precomp(p->w[k], q);
        p->wi[k] = nq_powmod(psiinv, e, q);
        p->wip[k] = nq_shoup_precomp(p->wi[k], q);
    }
    p->ninv = nq_invmod(N, q);
    p->ninvp = nq_shoup_precomp(p->ninv, q);
    p->br = nq_barrett_make(q);
    return 0;
}

static inline void nq_plan_free(nq_plan* p) {
    free(p->w);
    memset(p, 0, sizeof(*p));
}

/* In place; a[j] in [0, q) in, out[i] in [0, q) bit-reversed. */
static inline void nq_forward(const nq_plan* p, uint64_t* a) {
    const uint64_t q = p->q;
    const uint32_t N = p->N;
    uint32_t t = N;
    for (uint32_t m = 1; m < N; m <<= 1) {
        t >>= 1;
        for (uint32_t i = 0; i < m; i++) {
            const uint64_t W = p->w[m + i], Wp = p->wp[m + i];
            uint64_t* x = a + 2 * i * t;
            uint64_t* y = x + t;
            for (uint32_t j = 0; j < t; j++) {
                uint64_t u = x[j];
                uint64_t v = nq_mulshoup(y[j], W, Wp, q);
                uint64_t s = u + v;
                x[j] = s >= q ? s - q : s;
                y[j] = u >= v ? u - v : u + q - v;
            }
        }
    }
}

/* In place; bit-reversed in, natural order out, scaled by N^-1. */
static inline void nq_inverse(const nq_plan* p, uint64_t* a) {
    const uint64_t q = p->q;
    const uint32_t N = p->N;
    uint32_t t = 1;
    for (uint32_t m = N; m > 1; m >>= 1) {
        const uint32_t h = m >> 1;
        for (uint32_t i = 0; i < h; i++) {
            const uint64_t W = p->wi[h + i], Wp = p->wip[h + i];
            uint64_t* x = a + 2 * i * t;
            uint64_t* y = x + t;
            for (uint32_t j = 0; j < t; j++) {
                uint64_t u = x[j], v = y[j];
                uint64_t s = u + v;
                x[j] = s >= q ? s - q : s;
                uint64_t d = u >= v ? u - v : u + q - v;
                y[j] = nq_mulshoup(d, W, Wp, q);
            }
        }
        t <<= 1;
    }
    for (uint32_t j = 0; j < N; j++) a[j] = nq_mulshoup(a[j], p->ninv, p->ninvp, q);
}

#endif /* YATFHE_ORACLE_NTT_Q_H */
