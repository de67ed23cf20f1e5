/*
 * pbs_oracle.c -- plain-C restatement of the reference's GINX/MP21 programmable
 * bootstrap and of the seeded key generation that feeds it.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the cpu_baseline and
 * reference legs of bench.py may call it, to check or time against; the shipped library
 * (yatfhe_gb300/) never links, loads or runs it.  Every function cites the reference source it restates
 * (paths relative to the reference project).  Torus values are carried in int64 and
 * brought back to the torus width T with sext(), which reproduces both the reference's
 * int32 wrap arithmetic (TORUS32) and its longModPow2 reductions (TORUS56).
 */
#define _GNU_SOURCE
#include "pbs_oracle.h"

#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ntt_q.h"

/* yatfhe/include/yatfhe/torus.h:151,157 */
#define Q_49P_T32 562941363486721ULL
#define Q_61P_T56 1945555039024054273ULL

/* ------------------------------------------------------------------ helpers */

/* longModPow2 (yatfhe/include/yatfhe/numeric.h:69-71): sign-extend the low `bits` bits. */
static inline int64_t sext(int64_t x, int bits) {
    const int sh = 64 - bits;
    return (int64_t)((uint64_t)x << sh) >> sh;
}

/* ------------------------------------------------------------------ RNG */

/*
 * ChaCha20 (RFC 8439 sec. 2.3) keyed as oracle/shim/seeded_csprng.cpp keys the
 * reference's ChaCha20Rng: key = (seed_lo, seed_hi, 0 x 6), counter 0, nonce (stream, 0).
 */
typedef struct {
    uint32_t state[16];
    uint32_t block[16];
    int pos;
} po_rng;

static inline uint32_t rotl32(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }

#define QR(a, b, c, d)                                                                  \
    do {                                                                                \
        x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 16);                            \
        x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 12);                            \
        x[a] += x[b]; x[d] ^= x[a]; x[d] = rotl32(x[d], 8);                             \
        x[c] += x[d]; x[b] ^= x[c]; x[b] = rotl32(x[b], 7);                             \
    } while (0)

static void rng_seed(po_rng* r, uint64_t seed, uint32_t stream) {
    static const uint32_t sigma[4] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
    for (int i = 0; i < 4; i++) r->state[i] = sigma[i];
    r->state[4] = (uint32_t)seed;
    r->state[5] = (uint32_t)(seed >> 32);
    for (int i = 6; i < 12; i++) r->state[i] = 0;
    r->state[12] = 0;
    r->state[13] = 0;
    r->state[14] = stream;
    r->state[15] = 0;
    r->pos = 16;
}

static void rng_refill(po_rng* r) {
    uint32_t x[16];
    memcpy(x, r->state, sizeof(x));
    for (int i = 0; i < 10; i++) {
        QR(0, 4, 8, 12); QR(1, 5, 9, 13); QR(2, 6, 10, 14); QR(3, 7, 11, 15);
        QR(0, 5, 10, 15); QR(1, 6, 11, 12); QR(2, 7, 8, 13); QR(3, 4, 9, 14);
    }
    for (int i = 0; i < 16; i++) r->block[i] = x[i] + r->state[i];
    if (++r->state[12] == 0) ++r->state[13];
    r->pos = 0;
}

static inline uint32_t rng_next(po_rng* r) {
    if (r->pos == 16) rng_refill(r);
    return r->block[r->pos++];
}

/*
 * std::uniform_int_distribution as libstdc++ (GCC 13) implements it for a generator
 * whose outputs span exactly 32 bits: ranges below 2^32 are "downscaled" with Lemire's
 * nearly-divisionless multiply-and-reject in 64-bit arithmetic; a range of exactly 2^32
 * takes one draw; wider ranges are "upscaled" by drawing the high part recursively and
 * one more word for the low part, rejecting overflow.  Both the int32 and the uint64
 * instantiations the reference uses reduce to this on the unsigned difference b - a.
 */
static uint32_t rng_nd32(po_rng* r, uint32_t range) {
    uint64_t product = (uint64_t)rng_next(r) * range;
    uint32_t low = (uint32_t)product;
    if (low < range) {
        uint32_t threshold = (uint32_t)(-range) % range;
        while (low < threshold) {
            product = (uint64_t)rng_next(r) * range;
            low = (uint32_t)product;
        }
    }
    return (uint32_t)(product >> 32);
}

static uint64_t rng_urange(po_rng* r, uint64_t urange) {
    if (urange < 0xFFFFFFFFull) return rng_nd32(r, (uint32_t)(urange + 1));
    if (urange == 0xFFFFFFFFull) return rng_next(r);
    uint64_t ret, tmp;
    do {
        tmp = (uint64_t)0x100000000ull * rng_urange(r, urange >> 32);
        ret = tmp + rng_next(r);
    } while (ret > urange || ret < tmp);
    return ret;
}

/* uniform over [a, b] for signed bounds (the two's-complement wrap is the library's). */
static inline int64_t rng_uniform_i64(po_rng* r, int64_t a, int64_t b) {
    return (int64_t)(rng_urange(r, (uint64_t)b - (uint64_t)a) + (uint64_t)a);
}

/* binaryDistrib(rng) (yatfhe/src/numeric.cpp:11) */
static inline int rng_binary(po_rng* r) { return (int)rng_urange(r, 1); }

/* genTUniformNoise (yatfhe/src/numeric.cpp:47-55) */
static int64_t rng_tuniform(po_rng* r, int b) {
    const int bits = b + 2;
    const uint64_t mask = bits >= 64 ? UINT64_MAX : ((uint64_t)1 << bits) - 1;
    uint64_t cand = rng_urange(r, mask);
    uint64_t low = cand & 1;
    cand = (cand >> 1) + low;
    return (int64_t)cand - ((int64_t)1 << b);
}

/* ------------------------------------------------------------------ context */

struct po_ctx {
    po_params p;
    int T;               /* torus bits */
    int L;               /* key / decomposition levels = l_approx */
    uint64_t q;          /* qNtt */
    nq_plan plan;
    po_rng rng;
    int have_rng;
    int32_t* lwe_s;      /* n */
    int32_t* rlwe_s;     /* k*N */
    uint64_t* rlwe_s_ntt;/* k*N */
    uint64_t* bsk;       /* [n][L][k+1][k+1][N] */
    int32_t* ksk;        /* [k*N][t][n+1] */
    uint64_t* wwl_cprime;/* WWL+24 key: [n][L][k+1][N] (allocated on first use) */
    uint64_t* wwl_s2;    /* [l][k+1][N] (also the s2 key of the lazy family) */
    int64_t* lazy_cprime;/* lazy key: [n][L][k+1][N] coefficient-domain torus (allocated on first use) */
    uint64_t* grp_bsk;   /* group-g key: [keys][l][k+1][k+1][N] NTT domain (allocated on first use) */
    int grp;             /* its group g (0: none) */
    /* when set, po_keygen also records its random samples here (po_keygen_samples) */
    int32_t* rec_bsk_noise;   /* [n][L][k+1][N] */
    uint64_t* rec_bsk_mask;   /* [n][L][k+1][k][N] */
    int32_t* rec_ksk_mask;    /* [kN][t][n] */
    int32_t* rec_ksk_noise;   /* [kN][t] */
    char err[256];
};

static int fail(po_ctx* c, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
    return -1;
}

const char* po_last_error(po_ctx* c) { return c->err; }
uint64_t po_qntt(po_ctx* c) { return c->q; }

static size_t bsk_words(const po_ctx* c) {
    const size_t k1 = (size_t)c->p.k + 1;
    return (size_t)c->p.n * c->L * k1 * k1 * c->p.N;
}
static size_t ksk_words(const po_ctx* c) {
    return (size_t)c->p.k * c->p.N * c->p.ks_level * (c->p.n + 1);
}

po_ctx* po_create(const po_params* p) {
    if (p->torus_bits != 32 && p->torus_bits != 56) return NULL;
    po_ctx* c = (po_ctx*)calloc(1, sizeof(po_ctx));
    if (!c) return NULL;
    c->p = *p;
    c->T = p->torus_bits;
    c->L = p->l_approx;
    c->q = c->T == 32 ? Q_49P_T32 : Q_61P_T56;
    if (nq_plan_init(&c->plan, (uint32_t)p->N, c->q) != 0) {
        free(c);
        return NULL;
    }
    c->lwe_s = (int32_t*)calloc((size_t)p->n, sizeof(int32_t));
    c->rlwe_s = (int32_t*)calloc((size_t)p->k * p->N, sizeof(int32_t));
    c->rlwe_s_ntt = (uint64_t*)calloc((size_t)p->k * p->N, sizeof(uint64_t));
    c->bsk = (uint64_t*)calloc(bsk_words(c), sizeof(uint64_t));
    c->ksk = (int32_t*)calloc(ksk_words(c), sizeof(int32_t));
    if (!c->lwe_s || !c->rlwe_s || !c->rlwe_s_ntt || !c->bsk || !c->ksk) {
        po_destroy(c);
        return NULL;
    }
    return c;
}

void po_destroy(po_ctx* c) {
    if (!c) return;
    nq_plan_free(&c->plan);
    free(c->lwe_s);
    free(c->rlwe_s);
    free(c->rlwe_s_ntt);
    free(c->bsk);
    free(c->ksk);
    free(c->wwl_cprime);
    free(c->wwl_s2);
    free(c->lazy_cprime);
    free(c->grp_bsk);
    free(c);
}

/* ------------------------------------------------------------------ ring helpers */

/* applyNtt (yatfhe/include/yatfhe/ntt_hexl.h:34-44): lift v < 0 to v + q, forward NTT. */
static void ntt_from_torus(const po_ctx* c, uint64_t* out, const int64_t* in) {
    const int N = c->p.N;
    for (int j = 0; j < N; j++) out[j] = in[j] < 0 ? (uint64_t)in[j] + c->q : (uint64_t)in[j];
    nq_forward(&c->plan, out);
}

/* applyIntt (yatfhe/src/ntt_hexl.cpp:153-175): inverse NTT, centre at (q+1)/2, reduce to T bits. */
static void intt_to_torus(const po_ctx* c, int64_t* out, uint64_t* in_scratch) {
    const int N = c->p.N;
    const uint64_t half = (c->q + 1) >> 1;
    nq_inverse(&c->plan, in_scratch);
    for (int j = 0; j < N; j++) {
        uint64_t r = in_scratch[j];
        uint64_t centred = r >= half ? r - c->q : r;
        out[j] = sext((int64_t)centred, c->T);
    }
}

static inline uint64_t addmod(uint64_t a, uint64_t b, uint64_t q) {
    uint64_t s = a + b;
    return s >= q ? s - q : s;
}

/* validateRotator (yatfhe/src/polynomial.cpp:22-29) */
static void validate_rotator(int* aTrue, int* isWrap, int a, int N) {
    int t = a % (2 * N);
    if (t < 0) t += 2 * N;
    *isWrap = t < N ? 1 : -1;
    *aTrue = t < N ? t : t - N;
}

/* rotateTorusPolynomial (yatfhe/src/polynomial.cpp:184-193) and
 * rotateTorusPolynomialMinusOne (:213-238): out = X^a in, or X^a in - in. */
static void rotate_poly(const po_ctx* c, int64_t* out, const int64_t* in, int a, int minus_one) {
    const int N = c->p.N;
    int aTrue, isWrap;
    validate_rotator(&aTrue, &isWrap, a, N);
    for (int i = 0; i < N; i++) {
        int64_t r = i < aTrue ? -in[i - aTrue + N] * isWrap : in[i - aTrue] * isWrap;
        out[i] = minus_one ? sext(r - in[i], c->T) : sext(r, c->T);
    }
}

/*
 * zeroMeanDigits (yatfhe/include/yatfhe/gadget_decomposition.h:76-95): signed balanced
 * digits of the top levels*radixBits bits of a widthBits-wide value, rounded half away
 * from zero, emitted from the least significant level up with a carry; ties go up when
 * the top bit of the next window is set.  digits[level], level 0 most significant.
 */
static void zero_mean_digits(uint64_t u, int levels, int radixBits, int widthBits, int64_t* digits) {
    const uint64_t wmask = widthBits >= 64 ? UINT64_MAX : (((uint64_t)1 << widthBits) - 1);
    u &= wmask;
    const int negative = (int)((u >> (widthBits - 1)) & 1);
    const int dropped = widthBits - levels * radixBits;
    const uint64_t bias = dropped > 0 ? (uint64_t)1 << (dropped - 1) : 0;
    const uint64_t m = (negative ? (0 - u) & wmask : u) + bias;
    const int64_t B = (int64_t)1 << radixBits, halfB = B >> 1;
    int64_t carry = 0;
    for (int level = levels - 1; level >= 0; --level) {
        const int shift = widthBits - (level + 1) * radixBits;
        const int64_t window = (int64_t)((m >> shift) & (uint64_t)(B - 1));
        const int64_t digit = window + carry;
        const int64_t tie = level > 0 ? (int64_t)((m >> (shift + 2 * radixBits - 1)) & 1) : 0;
        carry = (digit > halfB) | ((digit == halfB) & tie);
        const int64_t bal = carry ? digit - B : digit;
        digits[level] = negative ? -bal : bal;
    }
}

/* modSwitchFromTorusGeneral (yatfhe/src/numeric.cpp:189-208), downscaling branch with a
 * power-of-two target: round half away from zero, then sign-extend. */
static int64_t modswitch_down(int64_t x, int fromBits, int toBits) {
    const int64_t scale = (int64_t)1 << (fromBits - toBits);
    const int64_t real = x >= 0 ? (x + scale / 2) / scale : (x - scale / 2) / scale;
    return sext(real, toBits);
}

static int log2i(int x) {
    int r = 0;
    while ((1 << r) < x) r++;
    return r;
}

/* ------------------------------------------------------------------ key generation */

/* NTT-domain RLWE encryption: initTrlweMultiSampleSimple / initTrlweSingleSampleSimple
 * (yatfhe/src/trlwe.cpp:24-46) then symEncTrlweNttSimple (:58-60).  `mu` holds the N
 * torus plaintext coefficients; out = [a_0..a_{k-1}, b] NTT polys. */
static void enc_trlwe_ntt(po_ctx* c, uint64_t* out, const int64_t* mu, int64_t* tmpT, int32_t* rec_noise,
                          uint64_t* rec_mask) {
    const int N = c->p.N, k = c->p.k;
    const uint64_t q = c->q;
    uint64_t* b = out + (size_t)k * N;
    for (int j = 0; j < N; j++) {
        const int64_t e = rng_tuniform(&c->rng, c->p.rlwe_noise_b);
        if (rec_noise) rec_noise[j] = (int32_t)e;
        tmpT[j] = sext(mu[j] + e, c->T);
    }
    ntt_from_torus(c, b, tmpT);
    for (int r = 0; r < k; r++)
        for (int j = 0; j < N; j++) out[(size_t)r * N + j] = rng_urange(&c->rng, q - 1);
    if (rec_mask) memcpy(rec_mask, out, sizeof(uint64_t) * (size_t)k * N);
    for (int r = 0; r < k; r++)
        for (int j = 0; j < N; j++)
            b[j] = addmod(b[j], nq_mulmod(&c->plan.br, out[(size_t)r * N + j], c->rlwe_s_ntt[(size_t)r * N + j]), q);
}

/* symEncTlwe (yatfhe/src/tlwe.cpp:21-31) with addTUniformNoise (numeric.cpp:57-60) and
 * addTorus / longModP mod LWE_Q = 2^32 (numeric.h:53-66,163-177). */
static void enc_tlwe(po_ctx* c, int32_t* out, int64_t message, const int32_t* s, int n, int32_t* rec_noise) {
    int64_t tmp = 0;
    for (int i = 0; i < n; i++) {
        int64_t a = rng_uniform_i64(&c->rng, -((int64_t)1 << 31), ((int64_t)1 << 31) - 1);
        out[i] = (int32_t)a;
        if (s[i]) tmp += a * s[i];
    }
    const int64_t e = rng_tuniform(&c->rng, c->p.lwe_noise_b);
    if (rec_noise) *rec_noise = (int32_t)e;
    int64_t muE = sext(message + e, 32);
    out[n] = (int32_t)sext(muE + sext(tmp, 32), 32);
}

/*
 * Keys from a seed, in the order oracle/ref_capi.cpp:ref_keygen draws them on one RNG
 * stream: genTlweKey (yatfhe/src/tlwe.cpp:10-18), genTrlweKey (yatfhe/src/trlwe.cpp:70-81),
 * encryptTrgswMPNtt(bsk[i], s_i, pos 0) for i = 0..n-1 (yatfhe/src/trgsw.cpp:36-51, the
 * per-i body of genBootstrappingKeyMP, bootstrapping.cpp:150-174), genTlweKeySwitchingKey
 * (yatfhe/src/keyswitching.cpp:19-29).
 */
/* genTlweKey (yatfhe/src/tlwe.cpp:10-18) and genTrlweKey (yatfhe/src/trlwe.cpp:70-81) on a
 * fresh stream 0 of `seed`; tmpT is N words of scratch. */
static void keygen_secrets(po_ctx* c, uint64_t seed, int64_t* tmpT) {
    const int n = c->p.n, N = c->p.N, k = c->p.k;
    rng_seed(&c->rng, seed, 0);
    c->have_rng = 1;
    for (int i = 0; i < n; i++) c->lwe_s[i] = rng_binary(&c->rng);
    for (int r = 0; r < k; r++) {
        for (int j = 0; j < N; j++) c->rlwe_s[(size_t)r * N + j] = rng_binary(&c->rng);
        for (int j = 0; j < N; j++) tmpT[j] = c->rlwe_s[(size_t)r * N + j];
        ntt_from_torus(c, c->rlwe_s_ntt + (size_t)r * N, tmpT);
    }
}

/* genTlweKeySwitchingKey (yatfhe/src/keyswitching.cpp:19-29):
 * ksk[i][j] = LWE_s(s'_i * 2^(32 - (j+1) ksRadix)). */
static void keygen_ksk(po_ctx* c) {
    const int kN = c->p.k * c->p.N, t = c->p.ks_level, n = c->p.n, nb = n + 1;
    for (int i = 0; i < kN; i++) {
        for (int j = 0; j < t; j++) {
            const int sh = 32 - (j + 1) * c->p.ks_radix_bits;
            const int64_t m = sext((int64_t)c->rlwe_s[i] << sh, c->T);
            int32_t* row = c->ksk + ((size_t)i * t + j) * nb;
            enc_tlwe(c, row, m, c->lwe_s, n, c->rec_ksk_noise ? c->rec_ksk_noise + (size_t)i * t + j : NULL);
            if (c->rec_ksk_mask) memcpy(c->rec_ksk_mask + ((size_t)i * t + j) * n, row, sizeof(int32_t) * n);
        }
    }
}

int po_keygen(po_ctx* c, uint64_t seed) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L, T = c->T;
    const int k1 = k + 1;
    int64_t* tmpT = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    int64_t* muPoly = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    uint64_t* muNtt = (uint64_t*)calloc((size_t)N, sizeof(uint64_t));
    int64_t* zeroPoly = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    if (!tmpT || !muPoly || !muNtt || !zeroPoly) {
        free(tmpT); free(muPoly); free(muNtt); free(zeroPoly);
        return fail(c, "po_keygen: out of memory");
    }
    keygen_secrets(c, seed, tmpT);
    const size_t rowWords = (size_t)k1 * N;           /* one RLWE sample */
    const size_t lvlWords = (size_t)k1 * rowWords;    /* c[lvl][0..k-1] + cPrime[lvl] */
    for (int i = 0; i < n; i++) {
        const int64_t mu = c->lwe_s[i];
        memset(muPoly, 0, sizeof(int64_t) * N);
        for (int lvl = 0; lvl < L; lvl++) {
            uint64_t* g = c->bsk + ((size_t)i * L + lvl) * lvlWords;
            muPoly[0] = sext(mu << (T - (lvl + 1) * c->p.radix_bits), T);
            ntt_from_torus(c, muNtt, muPoly);
            const size_t rec = ((size_t)i * L + lvl) * k1;  /* recorded row index, row k = cPrime */
            /* cPrime[lvl] = RLWE(mu * g_lvl) */
            enc_trlwe_ntt(c, g + (size_t)k * rowWords, muPoly, tmpT,
                          c->rec_bsk_noise ? c->rec_bsk_noise + (rec + k) * N : NULL,
                          c->rec_bsk_mask ? c->rec_bsk_mask + (rec + k) * k * N : NULL);
            /* c[lvl][r] = RLWE(0) with a[r] += NTT(mu * g_lvl) */
            for (int r = 0; r < k; r++) {
                uint64_t* row = g + (size_t)r * rowWords;
                enc_trlwe_ntt(c, row, zeroPoly, tmpT, c->rec_bsk_noise ? c->rec_bsk_noise + (rec + r) * N : NULL,
                              c->rec_bsk_mask ? c->rec_bsk_mask + (rec + r) * k * N : NULL);
                for (int j = 0; j < N; j++) row[(size_t)r * N + j] = addmod(row[(size_t)r * N + j], muNtt[j], c->q);
            }
        }
    }
    keygen_ksk(c);
    free(tmpT);
    free(muPoly);
    free(muNtt);
    free(zeroPoly);
    return 0;
}

int po_encrypt(po_ctx* c, const int64_t* mu, int count, int32_t* out) {
    if (!c->have_rng) return fail(c, "po_encrypt: no RNG stream (run po_keygen first)");
    const int n = c->p.n;
    for (int i = 0; i < count; i++) enc_tlwe(c, out + (size_t)i * (n + 1), mu[i], c->lwe_s, n, NULL);
    return 0;
}

/* po_encrypt with each ciphertext's random samples written out: mask [count][n] (the
 * uniform a_i) and noise [count] (the TUniform(lwe_noise_b) error of b). */
int po_encrypt_samples(po_ctx* c, const int64_t* mu, int count, int32_t* out, int32_t* mask, int32_t* noise) {
    if (!c->have_rng) return fail(c, "po_encrypt_samples: no RNG stream (run po_keygen first)");
    const int n = c->p.n;
    for (int i = 0; i < count; i++) {
        int32_t* row = out + (size_t)i * (n + 1);
        enc_tlwe(c, row, mu[i], c->lwe_s, n, noise + i);
        memcpy(mask + (size_t)i * n, row, sizeof(int32_t) * n);
    }
    return 0;
}

/* symEncTrlweMultiSampleSimple (yatfhe/src/trlwe.cpp:40-47,62-64: initTrlweMultiSampleSimple
 * then symEncTrlweNttSimple) of `count` torus polynomials mu [count][N] into NTT-domain
 * samples out [count][k+1][N] (a_0 .. a_{k-1}, b), each sample's TUniform(rlwe_noise_b)
 * noise [count][N] and uniform masks [count][k][N] written out. */
int po_encrypt_rlwe_ntt_samples(po_ctx* c, const int64_t* mu, int count, uint64_t* out, uint64_t* mask,
                                int32_t* noise) {
    if (!c->have_rng) return fail(c, "po_encrypt_rlwe_ntt_samples: no RNG stream (run po_keygen first)");
    const int N = c->p.N, k = c->p.k;
    int64_t* tmpT = (int64_t*)malloc(sizeof(int64_t) * N);
    if (!tmpT) return fail(c, "po_encrypt_rlwe_ntt_samples: out of memory");
    for (int i = 0; i < count; i++)
        enc_trlwe_ntt(c, out + (size_t)i * (k + 1) * N, mu + (size_t)i * N, tmpT, noise + (size_t)i * N,
                      mask + (size_t)i * k * N);
    free(tmpT);
    return 0;
}

/* symDecTlweToInt (yatfhe/src/tlwe.cpp:44-53) with roundTorusGeneralError (numeric.cpp:95-98)
 * and modSwitchToTorusGeneral (numeric.cpp:182-187), all mod LWE_Q = 2^32. */
static int64_t int_mod_p(int64_t a, int64_t p) {
    int64_t b = a % p;
    if (b > (p - 1) / 2) b -= p;
    else if (b < -p / 2) b += p;
    return b;
}

static int64_t modswitch_general(int64_t x, int64_t newMod) {
    const int64_t torusQ = (int64_t)1 << 32;
    const int64_t scale = torusQ / newMod;
    const int64_t real = x >= 0 ? (x + scale / 2) / scale : (x - scale / 2) / scale;
    /* longModP: pow2 -> sign-extend, else centred remainder */
    if ((newMod & (newMod - 1)) == 0) return sext(real, log2i((int)newMod));
    return int_mod_p(real, newMod);
}

int po_decrypt(po_ctx* c, const int32_t* in, int count, int base, int32_t* out) {
    const int n = c->p.n;
    for (int ci = 0; ci < count; ci++) {
        const int32_t* x = in + (size_t)ci * (n + 1);
        int64_t tmp = 0;
        for (int i = 0; i < n; i++)
            if (c->lwe_s[i]) tmp += (int64_t)x[i] * c->lwe_s[i];
        int64_t phase = sext((int64_t)x[n] - sext(tmp, 32), 32);
        int64_t t = modswitch_general(phase, base);
        int64_t rounded = int_mod_p(t, base) * (((int64_t)1 << 32) / base);
        out[ci] = (int32_t)modswitch_general(sext(rounded, 32), base);
    }
    return 0;
}

int po_get_keys(po_ctx* c, int32_t* lwe_s, int32_t* rlwe_s) {
    memcpy(lwe_s, c->lwe_s, sizeof(int32_t) * c->p.n);
    memcpy(rlwe_s, c->rlwe_s, sizeof(int32_t) * c->p.k * c->p.N);
    return 0;
}

int po_set_keys(po_ctx* c, const int32_t* lwe_s, const int32_t* rlwe_s) {
    const int N = c->p.N;
    memcpy(c->lwe_s, lwe_s, sizeof(int32_t) * c->p.n);
    memcpy(c->rlwe_s, rlwe_s, sizeof(int32_t) * c->p.k * N);
    int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * N);
    if (!tmp) return fail(c, "po_set_keys: out of memory");
    for (int r = 0; r < c->p.k; r++) {
        for (int j = 0; j < N; j++) tmp[j] = rlwe_s[(size_t)r * N + j];
        ntt_from_torus(c, c->rlwe_s_ntt + (size_t)r * N, tmp);
    }
    free(tmp);
    return 0;
}

int po_get_ksk(po_ctx* c, int32_t* out) { memcpy(out, c->ksk, sizeof(int32_t) * ksk_words(c)); return 0; }
int po_set_ksk(po_ctx* c, const int32_t* in) { memcpy(c->ksk, in, sizeof(int32_t) * ksk_words(c)); return 0; }
int po_get_bsk_ntt(po_ctx* c, uint64_t* out) { memcpy(out, c->bsk, sizeof(uint64_t) * bsk_words(c)); return 0; }
int po_set_bsk_ntt(po_ctx* c, const uint64_t* in) { memcpy(c->bsk, in, sizeof(uint64_t) * bsk_words(c)); return 0; }

/* ------------------------------------------------------------------ BSK file */

/*
 * serializeBskMP / deserializeBskMP (yatfhe/src/ya_serializer.cpp:276-303) with the
 * nested serializers for TrgswMPDft (:176-218), TrlweDft (:76-98) and NttPolynomial
 * (:21-30): native-endian PODs, int = 4 bytes, bool = 1 byte.
 */
static int wr(FILE* f, const void* p, size_t n) { return fwrite(p, 1, n, f) == n ? 0 : -1; }
static int rd(FILE* f, void* p, size_t n) { return fread(p, 1, n, f) == n ? 0 : -1; }

static int wr_trlwe_dft(FILE* f, const uint64_t* rows, int k, int N) {
    int32_t kk = k;
    uint8_t init = 1;
    int32_t NN = N, asz = k;
    int e = 0;
    e |= wr(f, &kk, 4);
    e |= wr(f, &init, 1);
    e |= wr(f, &NN, 4);
    e |= wr(f, rows + (size_t)k * N, sizeof(uint64_t) * N); /* b */
    e |= wr(f, &asz, 4);
    for (int r = 0; r < k; r++) {
        e |= wr(f, &NN, 4);
        e |= wr(f, rows + (size_t)r * N, sizeof(uint64_t) * N);
    }
    return e;
}

static int rd_expect_i32(FILE* f, int32_t want) {
    int32_t v;
    if (rd(f, &v, 4)) return -1;
    return v == want ? 0 : -1;
}

static int rd_trlwe_dft(FILE* f, uint64_t* rows, int k, int N) {
    uint8_t init;
    if (rd_expect_i32(f, k) || rd(f, &init, 1) || init != 1) return -1;
    if (rd_expect_i32(f, N) || rd(f, rows + (size_t)k * N, sizeof(uint64_t) * N)) return -1;
    if (rd_expect_i32(f, k)) return -1;
    for (int r = 0; r < k; r++)
        if (rd_expect_i32(f, N) || rd(f, rows + (size_t)r * N, sizeof(uint64_t) * N)) return -1;
    return 0;
}

int po_save_bsk_file(po_ctx* c, const char* path) {
    FILE* f = fopen(path, "wb");
    if (!f) return fail(c, "po_save_bsk_file: cannot open %s", path);
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L;
    const size_t rowWords = (size_t)(k + 1) * N, lvlWords = (size_t)(k + 1) * rowWords;
    int e = 0;
    for (int i = 0; i < n; i++) {
        int32_t l = L, kk = k;
        uint8_t half = 0;
        e |= wr(f, &l, 4);
        e |= wr(f, &kk, 4);
        e |= wr(f, &half, 1);
        e |= wr(f, &l, 4);
        for (int lvl = 0; lvl < L; lvl++) {
            e |= wr(f, &kk, 4);
            for (int r = 0; r < k; r++)
                e |= wr_trlwe_dft(f, c->bsk + ((size_t)i * L + lvl) * lvlWords + r * rowWords, k, N);
        }
        e |= wr(f, &l, 4);
        for (int lvl = 0; lvl < L; lvl++)
            e |= wr_trlwe_dft(f, c->bsk + ((size_t)i * L + lvl) * lvlWords + (size_t)k * rowWords, k, N);
    }
    int32_t nn = n, group = 1;
    uint8_t half = 0;
    e |= wr(f, &nn, 4);
    e |= wr(f, &group, 4);
    e |= wr(f, &half, 1);
    if (fclose(f) != 0) e = -1;
    return e ? fail(c, "po_save_bsk_file: write failed") : 0;
}

int po_load_bsk_file(po_ctx* c, const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) return fail(c, "po_load_bsk_file: cannot open %s", path);
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L;
    const size_t rowWords = (size_t)(k + 1) * N, lvlWords = (size_t)(k + 1) * rowWords;
    int e = 0;
    for (int i = 0; i < n && !e; i++) {
        uint8_t half;
        e |= rd_expect_i32(f, L) | rd_expect_i32(f, k) | rd(f, &half, 1);
        if (e || half) { e = -1; break; }
        e |= rd_expect_i32(f, L);
        for (int lvl = 0; lvl < L && !e; lvl++) {
            e |= rd_expect_i32(f, k);
            for (int r = 0; r < k && !e; r++)
                e |= rd_trlwe_dft(f, c->bsk + ((size_t)i * L + lvl) * lvlWords + r * rowWords, k, N);
        }
        e |= rd_expect_i32(f, L);
        for (int lvl = 0; lvl < L && !e; lvl++)
            e |= rd_trlwe_dft(f, c->bsk + ((size_t)i * L + lvl) * lvlWords + (size_t)k * rowWords, k, N);
    }
    if (!e) e |= rd_expect_i32(f, n);
    fclose(f);
    return e ? fail(c, "po_load_bsk_file: %s is not a GINX key for these parameters", path) : 0;
}

/* ------------------------------------------------------------------ small pieces */

/* generateTestPolynomial (kind 0) / generateTestPolynomialFR (kind 1)
 * (yatfhe/src/polynomial.cpp:75-107) with modQ = 2N; slot values via
 * modSwitchToTorus32 (numeric.cpp:210-214) with TORUS_Q = 2^T. */
int po_test_polynomial(po_ctx* c, int kind, int modP, int64_t* v) {
    const int N = c->p.N, modQ = 2 * N;
    const int box = modQ / modP, half = box / 2, hh = half / 2;
    const int width = kind == 0 ? box : half;
    const int neg = kind == 0 ? half : hh;
    const int64_t scale = ((int64_t)1 << c->T) / modP;
    int64_t* t = (int64_t*)malloc(sizeof(int64_t) * N);
    if (!t) return fail(c, "po_test_polynomial: out of memory");
    for (int i = 0; i < N; i++) t[i] = sext(int_mod_p(i / width, modP) * scale, c->T);
    for (int i = 0; i < neg; i++) t[i] = sext(-t[i], c->T);
    for (int i = 0; i < N; i++) v[i] = t[(i + neg) % N]; /* std::rotate left by neg */
    free(t);
    return 0;
}

/* rescaleTlweToNewMod (yatfhe/src/tlwe.cpp:75-81) into mod 2N. */
int po_modswitch(po_ctx* c, const int32_t* in, int32_t* out) {
    const int n = c->p.n, bits = log2i(2 * c->p.N);
    for (int i = 0; i <= n; i++) out[i] = (int32_t)modswitch_down(in[i], 32, bits);
    return 0;
}

int po_rotate(po_ctx* c, const int64_t* in, int a, int minus_one, int64_t* out) {
    rotate_poly(c, out, in, a, minus_one);
    return 0;
}

/* decomposeRow (yatfhe/include/yatfhe/gadget_decomposition.h:190-236); out = [level][N]. */
int po_decompose(po_ctx* c, const int64_t* in, int levels, int64_t* out) {
    const int N = c->p.N;
    if (levels * c->p.radix_bits > c->T) return fail(c, "po_decompose: l * radixBits exceeds the torus width");
    int64_t d[64];
    for (int j = 0; j < N; j++) {
        zero_mean_digits((uint64_t)in[j], levels, c->p.radix_bits, c->T, d);
        for (int l = 0; l < levels; l++) out[(size_t)l * N + j] = d[l];
    }
    return 0;
}

/* signedGadgetDecompositionKs (yatfhe/src/gadget_decomposition.cpp:53-56). */
int po_decompose_ks(po_ctx* c, int64_t value, int64_t* out) {
    zero_mean_digits((uint64_t)value, c->p.ks_level, c->p.ks_radix_bits, 32, out);
    return 0;
}

int po_ntt_forward(po_ctx* c, const int64_t* in, uint64_t* out) {
    ntt_from_torus(c, out, in);
    return 0;
}

int po_ntt_inverse(po_ctx* c, const uint64_t* in, int64_t* out) {
    uint64_t* t = (uint64_t*)malloc(sizeof(uint64_t) * c->p.N);
    if (!t) return fail(c, "po_ntt_inverse: out of memory");
    memcpy(t, in, sizeof(uint64_t) * c->p.N);
    intt_to_torus(c, out, t);
    free(t);
    return 0;
}

/* ------------------------------------------------------------------ external product */

typedef struct {
    int64_t* digits;   /* L x N */
    uint64_t* dntt;    /* N */
    uint64_t* acc;     /* (k+1) x N, NTT domain */
    int64_t* tmp;      /* (k+1) x N, torus */
    int64_t* dg;       /* per-value digit scratch, L */
} ep_scratch;

static int ep_alloc(const po_ctx* c, ep_scratch* s) {
    const int N = c->p.N, k1 = c->p.k + 1;
    s->digits = (int64_t*)malloc(sizeof(int64_t) * (size_t)c->L * N);
    s->dntt = (uint64_t*)malloc(sizeof(uint64_t) * N);
    s->acc = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)k1 * N);
    s->tmp = (int64_t*)malloc(sizeof(int64_t) * (size_t)k1 * N);
    s->dg = (int64_t*)malloc(sizeof(int64_t) * (size_t)(c->L > 0 ? c->L : 1));
    return (s->digits && s->dntt && s->acc && s->tmp && s->dg) ? 0 : -1;
}

static void ep_free(ep_scratch* s) {
    free(s->digits); free(s->dntt); free(s->acc); free(s->tmp); free(s->dg);
}

/*
 * externalProductTrgswMPNttImpl (yatfhe/src/trgsw.cpp:712-767): decompose every input
 * poly into L levels (gadgetDecomposeTrlwe, yatfhe/src/trlwe.cpp:185-198), NTT each
 * digit poly, multiply-accumulate against the key rows -- a-digits against c[lvl][r],
 * b-digits against cPrime[lvl] (:737-744) -- sum all levels mod q, inverse NTT (:761-766).
 * The NTT-domain sum is a sum mod q, so accumulating every (level, row) product into one
 * accumulator gives the same residues as the reference's per-level partials.
 * in/out = [a_0..a_{k-1}, b], may alias.
 */
static void external_product(const po_ctx* c, ep_scratch* s, const uint64_t* key, const int64_t* in, int64_t* out) {
    const int N = c->p.N, k = c->p.k, k1 = k + 1, L = c->L;
    const uint64_t q = c->q;
    const nq_barrett* br = &c->plan.br;
    const size_t rowWords = (size_t)k1 * N, lvlWords = (size_t)k1 * rowWords;
    memset(s->acc, 0, sizeof(uint64_t) * rowWords);
    for (int r = 0; r < k1; r++) {
        const int64_t* poly = in + (size_t)r * N;
        for (int j = 0; j < N; j++) {
            zero_mean_digits((uint64_t)poly[j], L, c->p.radix_bits, c->T, s->dg);
            for (int lvl = 0; lvl < L; lvl++) s->digits[(size_t)lvl * N + j] = s->dg[lvl];
        }
        for (int lvl = 0; lvl < L; lvl++) {
            ntt_from_torus(c, s->dntt, s->digits + (size_t)lvl * N);
            const uint64_t* keyRow = key + (size_t)lvl * lvlWords + (size_t)r * rowWords;
            for (int o = 0; o < k1; o++) {
                const uint64_t* kp = keyRow + (size_t)o * N;
                uint64_t* ap = s->acc + (size_t)o * N;
                for (int j = 0; j < N; j++) ap[j] = addmod(ap[j], nq_mulmod(br, s->dntt[j], kp[j]), q);
            }
        }
    }
    for (int o = 0; o < k1; o++) intt_to_torus(c, out + (size_t)o * N, s->acc + (size_t)o * N);
}

int po_external_product(po_ctx* c, const int64_t* in, int i, int64_t* out) {
    ep_scratch s;
    if (ep_alloc(c, &s)) { ep_free(&s); return fail(c, "po_external_product: out of memory"); }
    const size_t k1 = (size_t)c->p.k + 1;
    external_product(c, &s, c->bsk + (size_t)i * c->L * k1 * k1 * c->p.N, in, out);
    ep_free(&s);
    return 0;
}

/* ------------------------------------------------------------------ blind rotation */

/* genNoiselessTrlweSample (yatfhe/src/trlwe.cpp:175-182) + the binary branch of
 * blindRotateMP21Ntt (yatfhe/src/blind_rotate.cpp:1556-1563):
 *   for i < n: if a_i != 0: acc += ExtProd(BSK_i, X^{a_i} acc - acc). */
static void blind_rotate(const po_ctx* c, ep_scratch* s, const int32_t* scaled, const int64_t* v, int64_t* acc,
                         const int* checkpoints, int ncheck, int64_t* acc_out) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, k1 = k + 1;
    const size_t stride = (size_t)k1 * N;
    const size_t keyWords = (size_t)c->L * k1 * k1 * N;
    memset(acc, 0, sizeof(int64_t) * (size_t)k * N);
    rotate_poly(c, acc + (size_t)k * N, v, -scaled[n], 0);
    int cp = 0;
    for (int i = 0; i < n; i++) {
        const int a = scaled[i];
        if (a != 0) {
            for (int r = 0; r < k1; r++) rotate_poly(c, s->tmp + (size_t)r * N, acc + (size_t)r * N, a, 1);
            external_product(c, s, c->bsk + (size_t)i * keyWords, s->tmp, s->tmp);
            for (size_t j = 0; j < stride; j++) acc[j] = sext(acc[j] + s->tmp[j], c->T);
        }
        while (cp < ncheck && checkpoints[cp] == i) {
            memcpy(acc_out + (size_t)cp * stride, acc, sizeof(int64_t) * stride);
            cp++;
        }
    }
}

/* extractTlweFromTrlwe(out, acc, 0) (yatfhe/src/trlwe.cpp:240-250): a'[r N + j] =
 * j == 0 ? a_r[0] : -a_r[N - j], b' = b[0], each rescaled 2^T -> 2^32 (numeric.cpp:189-208). */
static void extract(const po_ctx* c, const int64_t* acc, int32_t* out) {
    const int N = c->p.N, k = c->p.k, T = c->T;
    for (int r = 0; r < k; r++)
        for (int j = 0; j < N; j++) {
            int64_t x = j == 0 ? acc[(size_t)r * N] : sext(-acc[(size_t)r * N + N - j], T);
            out[(size_t)r * N + j] = (int32_t)modswitch_down(x, T, 32);
        }
    out[(size_t)k * N] = (int32_t)modswitch_down(acc[(size_t)k * N], T, 32);
}

/* switchKeyForTlwe (yatfhe/src/keyswitching.cpp:48-72): int64 sums of digit * ksk word,
 * zero digits skipped, results reduced mod 2^32. */
static void keyswitch(const po_ctx* c, const int32_t* in, int32_t* out, int64_t* delta) {
    const int n = c->p.n, kN = c->p.k * c->p.N, t = c->p.ks_level, nb = n + 1;
    int64_t d[64];
    memset(delta, 0, sizeof(int64_t) * nb);
    for (int i = 0; i < kN; i++) {
        zero_mean_digits((uint64_t)(int64_t)in[i], t, c->p.ks_radix_bits, 32, d);
        for (int j = 0; j < t; j++) {
            const int64_t coef = d[j];
            if (!coef) continue;
            const int32_t* row = c->ksk + ((size_t)i * t + j) * nb;
            for (int x = 0; x < nb; x++) delta[x] += coef * row[x];
        }
    }
    for (int x = 0; x < n; x++) out[x] = (int32_t)sext(-delta[x], 32);
    out[n] = (int32_t)sext((int64_t)in[kN] - delta[n], 32);
}

int po_extract(po_ctx* c, const int64_t* acc, int32_t* out) {
    extract(c, acc, out);
    return 0;
}

int po_keyswitch(po_ctx* c, const int32_t* in, int32_t* out) {
    int64_t* delta = (int64_t*)malloc(sizeof(int64_t) * (c->p.n + 1));
    if (!delta) return fail(c, "po_keyswitch: out of memory");
    keyswitch(c, in, out, delta);
    free(delta);
    return 0;
}

int po_blind_rotate_trace(po_ctx* c, const int32_t* in, const int64_t* v, const int* checkpoints, int ncheck,
                          int64_t* acc_out, int64_t* acc_final) {
    ep_scratch s;
    if (ep_alloc(c, &s)) { ep_free(&s); return fail(c, "po_blind_rotate_trace: out of memory"); }
    int32_t* scaled = (int32_t*)malloc(sizeof(int32_t) * (c->p.n + 1));
    if (!scaled) { ep_free(&s); return fail(c, "po_blind_rotate_trace: out of memory"); }
    po_modswitch(c, in, scaled);
    blind_rotate(c, &s, scaled, v, acc_final, checkpoints, ncheck, acc_out);
    free(scaled);
    ep_free(&s);
    return 0;
}

/* ------------------------------------------------------------------ full bootstrap */

typedef struct {
    po_ctx* c;
    const int32_t* in;
    const int64_t* v;
    int32_t* out;
    int begin, end;
    int lazy;  /* 1: blindRotateLazyPipeAltNtt on the lazy key, 2: blindRotateNtt on the group key,
                  3: blindRotateLazyPipeAltNoFirstNtt on the lazy key */
    int rc;
} pbs_job;

static int blind_rotate_lazy(const po_ctx* c, ep_scratch* s, const int32_t* scaled, const int64_t* v, int64_t* acc,
                             int no_first);
static int blind_rotate_group(const po_ctx* c, const int32_t* scaled, const int64_t* v, int64_t* acc);

/* functionalBootstrappingMPNtt (yatfhe/src/bootstrapping.cpp:71-80). */
static void* pbs_worker(void* arg) {
    pbs_job* j = (pbs_job*)arg;
    po_ctx* c = j->c;
    const int n = c->p.n, N = c->p.N, k = c->p.k, nb = n + 1;
    ep_scratch s;
    int32_t* scaled = (int32_t*)malloc(sizeof(int32_t) * nb);
    int64_t* acc = (int64_t*)malloc(sizeof(int64_t) * (size_t)(k + 1) * N);
    int32_t* ext = (int32_t*)malloc(sizeof(int32_t) * ((size_t)k * N + 1));
    int64_t* delta = (int64_t*)malloc(sizeof(int64_t) * nb);
    if (ep_alloc(c, &s) || !scaled || !acc || !ext || !delta) {
        j->rc = -1;
    } else {
        j->rc = 0;
        for (int i = j->begin; i < j->end; i++) {
            po_modswitch(c, j->in + (size_t)i * nb, scaled);
            if (j->lazy == 2) {
                if (blind_rotate_group(c, scaled, j->v, acc)) { j->rc = -1; break; }
            } else if (j->lazy) {
                if (blind_rotate_lazy(c, &s, scaled, j->v, acc, j->lazy == 3)) { j->rc = -1; break; }
            } else {
                blind_rotate(c, &s, scaled, j->v, acc, NULL, 0, NULL);
            }
            extract(c, acc, ext);
            keyswitch(c, ext, j->out + (size_t)i * nb, delta);
        }
    }
    ep_free(&s);
    free(scaled); free(acc); free(ext); free(delta);
    return NULL;
}

static int pbs_run(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads, int lazy) {
    if (threads < 1) threads = 1;
    if (threads > count) threads = count > 0 ? count : 1;
    pbs_job* jobs = (pbs_job*)calloc((size_t)threads, sizeof(pbs_job));
    pthread_t* tids = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    if (!jobs || !tids) { free(jobs); free(tids); return fail(c, "po_pbs: out of memory"); }
    int rc = 0;
    for (int t = 0; t < threads; t++) {
        jobs[t].c = c; jobs[t].in = in; jobs[t].v = v; jobs[t].out = out; jobs[t].lazy = lazy;
        jobs[t].begin = (int)((long long)count * t / threads);
        jobs[t].end = (int)((long long)count * (t + 1) / threads);
        if (threads == 1) pbs_worker(&jobs[t]);
        else if (pthread_create(&tids[t], NULL, pbs_worker, &jobs[t]) != 0) { jobs[t].rc = -1; tids[t] = 0; }
    }
    if (threads > 1)
        for (int t = 0; t < threads; t++)
            if (tids[t]) pthread_join(tids[t], NULL);
    for (int t = 0; t < threads; t++) rc |= jobs[t].rc;
    free(jobs);
    free(tids);
    return rc ? fail(c, "po_pbs: worker failed") : 0;
}

int po_pbs(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads) {
    return pbs_run(c, in, count, v, out, threads, 0);
}

/* ------------------------------------------------------------------ WWL+24 keys */

static size_t wwl_cprime_words(const po_ctx* c) {
    return (size_t)c->p.n * c->L * (c->p.k + 1) * c->p.N;
}
static size_t wwl_s2_words(const po_ctx* c) { return (size_t)c->p.l * (c->p.k + 1) * c->p.N; }

static int wwl_alloc(po_ctx* c) {
    if (!c->wwl_cprime) c->wwl_cprime = (uint64_t*)calloc(wwl_cprime_words(c), sizeof(uint64_t));
    if (!c->wwl_s2) c->wwl_s2 = (uint64_t*)calloc(wwl_s2_words(c), sizeof(uint64_t));
    return c->wwl_cprime && c->wwl_s2 ? 0 : -1;
}

/* uniformTorusDistrib(TORUS_MIN, TORUS_MAX) (yatfhe/src/numeric.cpp:223-227), TORUS_MIN/MAX =
 * -2^(T-1) and 2^(T-1)-1 (yatfhe/src/initializer.cpp:56-57). */
static inline int64_t rng_torus(po_ctx* c) {
    return rng_uniform_i64(&c->rng, -((int64_t)1 << (c->T - 1)), ((int64_t)1 << (c->T - 1)) - 1);
}

/* multTorusPolynomialAcc (yatfhe/src/polynomial.cpp:355-368): res += a * s, negacyclic, mod 2^T
 * (the int64 accumulator only ever matters mod 2^T, so it is kept as a wrapping uint64). */
static void mult_torus_acc(const po_ctx* c, int64_t* res, const int64_t* a, const int32_t* s) {
    const int N = c->p.N;
    for (int i = 0; i < N; i++) {
        uint64_t t = 0;
        for (int j = 0; j < N; j++) {
            const uint64_t prod = (uint64_t)a[j] * (uint64_t)(int64_t)(j <= i ? s[i - j] : s[N + i - j]);
            t = j <= i ? t + prod : t - prod;
        }
        res[i] = sext((int64_t)((uint64_t)res[i] + t), c->T);
    }
}

/*
 * symEncTrlweMultiSampleNtt (yatfhe/src/trlwe.cpp:103-106): initTrlweMultiSample (:32-38) draws
 * b = mu + TUniform noise, then the masks a[r] uniformly on the torus; symEncTrlweNtt (:53-57)
 * keeps the NTT-domain sample (NTT(a), NTT(b) + NTT(a) . NTT(s)) mod q.  out = [a_0..a_{k-1}, b].
 */
static void enc_trlwe_coef_ntt(po_ctx* c, uint64_t* out, const int64_t* mu, int64_t* tmpT) {
    const int N = c->p.N, k = c->p.k;
    uint64_t* b = out + (size_t)k * N;
    for (int j = 0; j < N; j++) tmpT[j] = sext(mu[j] + rng_tuniform(&c->rng, c->p.rlwe_noise_b), c->T);
    ntt_from_torus(c, b, tmpT);
    for (int r = 0; r < k; r++) {
        for (int j = 0; j < N; j++) tmpT[j] = rng_torus(c);
        ntt_from_torus(c, out + (size_t)r * N, tmpT);
    }
    for (int r = 0; r < k; r++)
        for (int j = 0; j < N; j++)
            b[j] = addmod(b[j], nq_mulmod(&c->plan.br, out[(size_t)r * N + j], c->rlwe_s_ntt[(size_t)r * N + j]), c->q);
}

/*
 * symEncTrlevWithKeyNtt(out, key, key.s, isPos = true) (yatfhe/src/trlev.cpp:75-96): l RLWE
 * encryptions of 0 in the coefficient domain (encTrlevSingleSample, :10-16, each one
 * symEncTrlweSingleSample = noise b, uniform masks, b += a s, trlwe.cpp:18-23,48-52,81-84),
 * then per level a[r] -= s_r 2^(T - (i+1) radix) and both polynomials to the NTT domain.
 * out = [l][a_0..a_{k-1}, b][N].
 */
static int enc_trlev_s(po_ctx* c, uint64_t* out) {
    const int N = c->p.N, k = c->p.k, l = c->p.l, T = c->T;
    const size_t row = (size_t)(k + 1) * N;
    int64_t* smp = (int64_t*)malloc(sizeof(int64_t) * row * l);
    if (!smp) return -1;
    for (int i = 0; i < l; i++) {
        int64_t* a = smp + (size_t)i * row;
        int64_t* b = a + (size_t)k * N;
        for (int j = 0; j < N; j++) b[j] = sext(rng_tuniform(&c->rng, c->p.rlwe_noise_b), T);
        for (int r = 0; r < k; r++)
            for (int j = 0; j < N; j++) a[(size_t)r * N + j] = rng_torus(c);
        for (int r = 0; r < k; r++) mult_torus_acc(c, b, a + (size_t)r * N, c->rlwe_s + (size_t)r * N);
    }
    for (int i = 0; i < l; i++) {
        int64_t* a = smp + (size_t)i * row;
        uint64_t* o = out + (size_t)i * row;
        ntt_from_torus(c, o + (size_t)k * N, a + (size_t)k * N);
        const int sh = T - (i + 1) * c->p.radix_bits;
        for (int r = 0; r < k; r++) {
            for (int j = 0; j < N; j++)
                a[(size_t)r * N + j] = sext(a[(size_t)r * N + j] - ((int64_t)c->rlwe_s[(size_t)r * N + j] << sh), T);
            ntt_from_torus(c, o + (size_t)r * N, a + (size_t)r * N);
        }
    }
    free(smp);
    return 0;
}

/*
 * WWL+24 keys from a seed, in the order oracle/ref_capi.cpp:ref_keygen_wwl24 draws them on one
 * stream: the LWE and RLWE secrets, then per i and level the half-TRGSW row
 * cPrime[i][lvl] = RLWE(s_i g_lvl) (the per-i body of genBootstrappingKeyWWL24,
 * yatfhe/src/bootstrapping.cpp:106-126), then the key s2 = RLev(-s . s) (enc_trlev_s), then
 * the key-switching key.
 */
int po_keygen_wwl24(po_ctx* c, uint64_t seed) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L, T = c->T;
    if (wwl_alloc(c)) return fail(c, "po_keygen_wwl24: out of memory");
    int64_t* tmpT = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    int64_t* muPoly = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    if (!tmpT || !muPoly) {
        free(tmpT); free(muPoly);
        return fail(c, "po_keygen_wwl24: out of memory");
    }
    keygen_secrets(c, seed, tmpT);
    const size_t row = (size_t)(k + 1) * N;
    for (int i = 0; i < n; i++) {
        memset(muPoly, 0, sizeof(int64_t) * N);
        for (int lvl = 0; lvl < L; lvl++) {
            muPoly[0] = sext((int64_t)c->lwe_s[i] << (T - (lvl + 1) * c->p.radix_bits), T);
            enc_trlwe_coef_ntt(c, c->wwl_cprime + ((size_t)i * L + lvl) * row, muPoly, tmpT);
        }
    }
    int rc = enc_trlev_s(c, c->wwl_s2);
    free(tmpT);
    free(muPoly);
    if (rc) return fail(c, "po_keygen_wwl24: out of memory");
    keygen_ksk(c);
    return 0;
}

int po_get_wwl24(po_ctx* c, uint64_t* cprime, uint64_t* s2) {
    if (!c->wwl_cprime || !c->wwl_s2) return fail(c, "po_get_wwl24: no WWL+24 key");
    memcpy(cprime, c->wwl_cprime, sizeof(uint64_t) * wwl_cprime_words(c));
    memcpy(s2, c->wwl_s2, sizeof(uint64_t) * wwl_s2_words(c));
    return 0;
}

int po_set_wwl24(po_ctx* c, const uint64_t* cprime, const uint64_t* s2) {
    if (wwl_alloc(c)) return fail(c, "po_set_wwl24: out of memory");
    memcpy(c->wwl_cprime, cprime, sizeof(uint64_t) * wwl_cprime_words(c));
    memcpy(c->wwl_s2, s2, sizeof(uint64_t) * wwl_s2_words(c));
    return 0;
}

/*
 * switchTrlweToSecretEmbeddingNtt (yatfhe/src/trgsw.cpp:861-905) for every key index and
 * level, written into the GINX key (c->bsk, [i][lvl][row][poly][N]): the mask polynomials of
 * cPrime[lvl] go back to the torus (applyIntt), decomposeRow splits them into l digit
 * polynomials, and
 *   c[lvl][k1].a[k2] = sum_l' NTT(d_l'(a_k1)) . s2[l'].a[k2] + cPrime[lvl].b,
 *   c[lvl][k1].b     = sum_l' NTT(d_l'(a_k1)) . s2[l'].b            (mod q);
 * row k is cPrime[lvl] itself.  These are the rows blindRotateWWL24Ntt hands to its external
 * product (yatfhe/src/blind_rotate.cpp:1394-1408), so the GINX bootstrap on this key is the
 * WWL+24 bootstrap.
 */
int po_wwl24_expand(po_ctx* c) {
    if (!c->wwl_cprime || !c->wwl_s2) return fail(c, "po_wwl24_expand: no WWL+24 key");
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L, Ls = c->p.l, T = c->T;
    const uint64_t q = c->q;
    const size_t row = (size_t)(k + 1) * N, lvlWords = (size_t)(k + 1) * row;
    uint64_t* scratch = (uint64_t*)malloc(sizeof(uint64_t) * N);
    int64_t* torus = (int64_t*)malloc(sizeof(int64_t) * N);
    int64_t* digits = (int64_t*)malloc(sizeof(int64_t) * (size_t)Ls * N);
    int64_t* dpoly = (int64_t*)malloc(sizeof(int64_t) * N);
    uint64_t* dntt = (uint64_t*)malloc(sizeof(uint64_t) * N);
    int64_t dg[64];
    if (!scratch || !torus || !digits || !dpoly || !dntt || Ls > 64) {
        free(scratch); free(torus); free(digits); free(dpoly); free(dntt);
        return fail(c, "po_wwl24_expand: out of memory");
    }
    for (int i = 0; i < n; i++) {
        for (int lvl = 0; lvl < L; lvl++) {
            const uint64_t* cp = c->wwl_cprime + ((size_t)i * L + lvl) * row;
            uint64_t* g = c->bsk + ((size_t)i * L + lvl) * lvlWords;
            memcpy(g + (size_t)k * row, cp, sizeof(uint64_t) * row);
            for (int k1 = 0; k1 < k; k1++) {
                uint64_t* out = g + (size_t)k1 * row;
                memset(out, 0, sizeof(uint64_t) * row);
                memcpy(scratch, cp + (size_t)k1 * N, sizeof(uint64_t) * N);
                intt_to_torus(c, torus, scratch);
                for (int j = 0; j < N; j++) {
                    zero_mean_digits((uint64_t)torus[j], Ls, c->p.radix_bits, T, dg);
                    for (int lv = 0; lv < Ls; lv++) digits[(size_t)lv * N + j] = dg[lv];
                }
                for (int lv = 0; lv < Ls; lv++) {
                    memcpy(dpoly, digits + (size_t)lv * N, sizeof(int64_t) * N);
                    ntt_from_torus(c, dntt, dpoly);
                    const uint64_t* s2 = c->wwl_s2 + (size_t)lv * row;
                    for (int poly = 0; poly <= k; poly++)
                        for (int j = 0; j < N; j++)
                            out[(size_t)poly * N + j] = addmod(out[(size_t)poly * N + j],
                                nq_mulmod(&c->plan.br, dntt[j], s2[(size_t)poly * N + j]), q);
                }
                for (int k2 = 0; k2 < k; k2++)
                    for (int j = 0; j < N; j++)
                        out[(size_t)k2 * N + j] = addmod(out[(size_t)k2 * N + j], cp[(size_t)k * N + j], q);
            }
        }
    }
    free(scratch); free(torus); free(digits); free(dpoly); free(dntt);
    return 0;
}

/*
 * serializeBskWWL24 / deserializeBskWWL24 (yatfhe/src/ya_serializer.cpp:220-246): n half
 * TrgswMPDft (`[int l][int k][bool isHalf = 1][int l]` + l TrlweDft, :176-218), the TrlevDft
 * s2 (`[int l][int l]` + l TrlweDft, :101-115), then `[int n][int group]`.
 */
int po_save_wwl24_file(po_ctx* c, const char* path) {
    if (!c->wwl_cprime || !c->wwl_s2) return fail(c, "po_save_wwl24_file: no WWL+24 key");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(c, "po_save_wwl24_file: cannot open %s", path);
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L, Ls = c->p.l;
    const size_t row = (size_t)(k + 1) * N;
    int e = 0;
    for (int i = 0; i < n; i++) {
        int32_t l = L, kk = k;
        uint8_t half = 1;
        e |= wr(f, &l, 4);
        e |= wr(f, &kk, 4);
        e |= wr(f, &half, 1);
        e |= wr(f, &l, 4);
        for (int lvl = 0; lvl < L; lvl++) e |= wr_trlwe_dft(f, c->wwl_cprime + ((size_t)i * L + lvl) * row, k, N);
    }
    int32_t ls = Ls;
    e |= wr(f, &ls, 4);
    e |= wr(f, &ls, 4);
    for (int lv = 0; lv < Ls; lv++) e |= wr_trlwe_dft(f, c->wwl_s2 + (size_t)lv * row, k, N);
    int32_t nn = n, group = 1;
    e |= wr(f, &nn, 4);
    e |= wr(f, &group, 4);
    if (fclose(f) != 0) e = -1;
    return e ? fail(c, "po_save_wwl24_file: write failed") : 0;
}

int po_load_wwl24_file(po_ctx* c, const char* path) {
    if (wwl_alloc(c)) return fail(c, "po_load_wwl24_file: out of memory");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(c, "po_load_wwl24_file: cannot open %s", path);
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L, Ls = c->p.l;
    const size_t row = (size_t)(k + 1) * N;
    int e = 0;
    for (int i = 0; i < n && !e; i++) {
        uint8_t half = 0;
        e |= rd_expect_i32(f, L) | rd_expect_i32(f, k) | rd(f, &half, 1);
        if (e || half != 1) { e = -1; break; }
        e |= rd_expect_i32(f, L);
        for (int lvl = 0; lvl < L && !e; lvl++) e |= rd_trlwe_dft(f, c->wwl_cprime + ((size_t)i * L + lvl) * row, k, N);
    }
    if (!e) e |= rd_expect_i32(f, Ls) | rd_expect_i32(f, Ls);
    for (int lv = 0; lv < Ls && !e; lv++) e |= rd_trlwe_dft(f, c->wwl_s2 + (size_t)lv * row, k, N);
    if (!e) e |= rd_expect_i32(f, n);
    fclose(f);
    return e ? fail(c, "po_load_wwl24_file: %s is not a WWL+24 key for these parameters", path) : 0;
}

/* ------------------------------------------------------------------ keygen samples */

/*
 * po_keygen with its random samples written out, in the layout of the GPU's key generation
 * entry point: lwe_s [n], rlwe_s [kN] (the secrets), bsk_noise [n][L][k+1][N] (the
 * TUniform noise of each RLWE sample's b, row k = cPrime), bsk_mask [n][L][k+1][k][N] (its
 * uniform NTT-domain masks), ksk_mask [kN][t][n] and ksk_noise [kN][t] (the key-switching
 * samples' masks and noise).  The keys themselves are left in the context as po_keygen
 * leaves them.
 */
int po_keygen_samples(po_ctx* c, uint64_t seed, int32_t* lwe_s, int32_t* rlwe_s, int32_t* bsk_noise,
                      uint64_t* bsk_mask, int32_t* ksk_mask, int32_t* ksk_noise) {
    c->rec_bsk_noise = bsk_noise;
    c->rec_bsk_mask = bsk_mask;
    c->rec_ksk_mask = ksk_mask;
    c->rec_ksk_noise = ksk_noise;
    const int rc = po_keygen(c, seed);
    c->rec_bsk_noise = NULL;
    c->rec_bsk_mask = NULL;
    c->rec_ksk_mask = NULL;
    c->rec_ksk_noise = NULL;
    if (rc) return rc;
    memcpy(lwe_s, c->lwe_s, sizeof(int32_t) * c->p.n);
    memcpy(rlwe_s, c->rlwe_s, sizeof(int32_t) * (size_t)c->p.k * c->p.N);
    return 0;
}

/* ------------------------------------------------------------------ lazy ("OURS") keys */

/*
 * The key of blindRotateLazyPipeAltNtt (BootstrappingKeyMPLazyPipeAlt,
 * yatfhe/include/yatfhe/bootstrapping.h:284-307): per key index i and level lvl the half
 * TRGSW row bskPrime[i].cPrime[lvl] = RLWE(s_i g_lvl) kept in the coefficient domain (TrgswMP,
 * torus words), and the s2 key RLev(-s . s) in the NTT domain (held in c->wwl_s2).
 * genBootstrappingKeyMPLazyPipeAlt (yatfhe/src/bootstrapping.cpp:322-339) encrypts each row
 * with encryptTrgswMP (yatfhe/src/trgsw.cpp:18-34), whose symEncTrlweMultiSampleNtt
 * (yatfhe/src/trlwe.cpp:56-60,103-106) draws the samples of the WWL+24 key generation in the
 * same order and keeps the coefficient-domain sample (a, applyIntt(NTT(b) + NTT(a) . NTT(s)));
 * the mask a equals applyIntt(NTT(a)).  So the lazy key of a seed is the WWL+24 key of that
 * seed with its cPrime rows taken back to the torus.
 */
static int lazy_alloc(po_ctx* c) {
    if (!c->lazy_cprime) c->lazy_cprime = (int64_t*)calloc(wwl_cprime_words(c), sizeof(int64_t));
    if (!c->wwl_s2) c->wwl_s2 = (uint64_t*)calloc(wwl_s2_words(c), sizeof(uint64_t));
    return c->lazy_cprime && c->wwl_s2 ? 0 : -1;
}

int po_keygen_lazy(po_ctx* c, uint64_t seed) {
    if (po_keygen_wwl24(c, seed)) return -1;
    const int N = c->p.N;
    uint64_t* scratch = (uint64_t*)malloc(sizeof(uint64_t) * N);
    if (lazy_alloc(c) || !scratch) {
        free(scratch);
        return fail(c, "po_keygen_lazy: out of memory");
    }
    const size_t polys = wwl_cprime_words(c) / N;
    for (size_t p = 0; p < polys; p++) {
        memcpy(scratch, c->wwl_cprime + p * N, sizeof(uint64_t) * N);
        intt_to_torus(c, c->lazy_cprime + p * N, scratch);
    }
    free(scratch);
    return 0;
}

int po_get_lazy(po_ctx* c, int64_t* cprime, uint64_t* s2) {
    if (!c->lazy_cprime || !c->wwl_s2) return fail(c, "po_get_lazy: no lazy key");
    memcpy(cprime, c->lazy_cprime, sizeof(int64_t) * wwl_cprime_words(c));
    memcpy(s2, c->wwl_s2, sizeof(uint64_t) * wwl_s2_words(c));
    return 0;
}

int po_set_lazy(po_ctx* c, const int64_t* cprime, const uint64_t* s2) {
    if (lazy_alloc(c)) return fail(c, "po_set_lazy: out of memory");
    const size_t words = wwl_cprime_words(c);
    for (size_t j = 0; j < words; j++) c->lazy_cprime[j] = sext(cprime[j], c->T);
    memcpy(c->wwl_s2, s2, sizeof(uint64_t) * wwl_s2_words(c));
    return 0;
}

/* serialize(TorusPolynomial) (yatfhe/src/ya_serializer.cpp:33-36): [int N] + N Torus words
 * (int32 for T = 32, int64 for T = 56). */
static int wr_torus_poly(FILE* f, const int64_t* v, int N, int T) {
    int32_t nn = N;
    int e = wr(f, &nn, 4);
    for (int j = 0; j < N && !e; j++) {
        if (T == 32) {
            int32_t w = (int32_t)v[j];
            e |= wr(f, &w, 4);
        } else {
            e |= wr(f, &v[j], 8);
        }
    }
    return e;
}

static int rd_torus_poly(FILE* f, int64_t* v, int N, int T) {
    int e = rd_expect_i32(f, N);
    for (int j = 0; j < N && !e; j++) {
        if (T == 32) {
            int32_t w;
            e |= rd(f, &w, 4);
            v[j] = w;
        } else {
            e |= rd(f, &v[j], 8);
            v[j] = sext(v[j], T);
        }
    }
    return e;
}

/*
 * serializeBskLazyPipeAlt / deserializeBskLazyPipeAlt (yatfhe/src/ya_serializer.cpp:445-481):
 * the TrlevDft s2 (`[int l][int l]` + l TrlweDft, :101-115), then n half TrgswMP
 * (`[int L][int k][bool isHalf = 1][int L]` + L Trlwe, :131-146; a Trlwe is
 * `[int k][int N]` + b + `[int k]` + a_0..a_{k-1}, each a TorusPolynomial, :57-63), then
 * `[int level = L][int group = 1]`.
 */
int po_save_lazy_file(po_ctx* c, const char* path) {
    if (!c->lazy_cprime || !c->wwl_s2) return fail(c, "po_save_lazy_file: no lazy key");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(c, "po_save_lazy_file: cannot open %s", path);
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L, Ls = c->p.l, T = c->T;
    const size_t row = (size_t)(k + 1) * N;
    int32_t ls = Ls, l32 = L, k32 = k, n32 = N;
    int e = wr(f, &ls, 4) | wr(f, &ls, 4);
    for (int lv = 0; lv < Ls; lv++) e |= wr_trlwe_dft(f, c->wwl_s2 + (size_t)lv * row, k, N);
    for (int i = 0; i < n && !e; i++) {
        uint8_t half = 1;
        e |= wr(f, &l32, 4) | wr(f, &k32, 4) | wr(f, &half, 1) | wr(f, &l32, 4);
        for (int lvl = 0; lvl < L && !e; lvl++) {
            const int64_t* t = c->lazy_cprime + ((size_t)i * L + lvl) * row;
            e |= wr(f, &k32, 4) | wr(f, &n32, 4);
            e |= wr_torus_poly(f, t + (size_t)k * N, N, T);
            e |= wr(f, &k32, 4);
            for (int r = 0; r < k; r++) e |= wr_torus_poly(f, t + (size_t)r * N, N, T);
        }
    }
    int32_t group = 1;
    e |= wr(f, &l32, 4) | wr(f, &group, 4);
    if (fclose(f) != 0) e = -1;
    return e ? fail(c, "po_save_lazy_file: write failed") : 0;
}

int po_load_lazy_file(po_ctx* c, const char* path) {
    if (lazy_alloc(c)) return fail(c, "po_load_lazy_file: out of memory");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(c, "po_load_lazy_file: cannot open %s", path);
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->L, Ls = c->p.l, T = c->T;
    const size_t row = (size_t)(k + 1) * N;
    int e = rd_expect_i32(f, Ls) | rd_expect_i32(f, Ls);
    for (int lv = 0; lv < Ls && !e; lv++) e |= rd_trlwe_dft(f, c->wwl_s2 + (size_t)lv * row, k, N);
    for (int i = 0; i < n && !e; i++) {
        uint8_t half = 0;
        e |= rd_expect_i32(f, L) | rd_expect_i32(f, k) | rd(f, &half, 1);
        if (e || half != 1) { e = -1; break; }
        e |= rd_expect_i32(f, L);
        for (int lvl = 0; lvl < L && !e; lvl++) {
            int64_t* t = c->lazy_cprime + ((size_t)i * L + lvl) * row;
            e |= rd_expect_i32(f, k) | rd_expect_i32(f, N);
            if (!e) e |= rd_torus_poly(f, t + (size_t)k * N, N, T);
            if (!e) e |= rd_expect_i32(f, k);
            for (int r = 0; r < k && !e; r++) e |= rd_torus_poly(f, t + (size_t)r * N, N, T);
        }
    }
    if (!e) e |= rd_expect_i32(f, L) | rd_expect_i32(f, 1);
    fclose(f);
    return e ? fail(c, "po_load_lazy_file: %s is not a lazy key for these parameters", path) : 0;
}

/*
 * blindRotateLazyPipeAltNtt (yatfhe/src/blind_rotate.cpp:995-1135; its split of the work into
 * pipelined stages and threads does not change a result) for one ciphertext, scaled = its
 * mask and body switched to mod 2N:
 *   derived = RLWE(v s_0) = INTT(sum_lvl gdV[lvl] . NTT(bskPrime[0].cPrime[lvl]))
 *     (deriveFirstComponentNtt, yatfhe/src/trgsw.cpp:929-955; gdV[lvl] = NTT of digit lvl of
 *     v, prepareGdV, :911-927),
 *   acc = X^(-b) ((X^(a_0) - 1) derived + (0, v))                       (:1117-1124),
 *   for i = 1 .. n-1 with a_i != 0: acc = acc [x] TRGSW_i in place
 *     (externalProductTrgswMPNttInPlace, yatfhe/src/trgsw.cpp:774-776).
 * TRGSW_i is built from bskPrime[i] for this ciphertext (stageA and stageB, :1036-1085): each
 * level's row is rotated, cP = (X^(a_i) - 1) cPrime[lvl] with cP.b[0] += g_lvl
 * (rotateTrlweMinusOneBPlusOne, yatfhe/src/trlwe.cpp:291-297), the masks go into l digit
 * polynomials (gadgetDecomposeTrlweA, yatfhe/src/trlwe.cpp:200-211), and with D_l' = NTT of
 * digit l' of cP.a_k1
 *   cPrime[lvl].a[k1] = sum_l' D_l' . NTT(2^(T - (l'+1) radix))   (the gadget recomposer)
 *   cPrime[lvl].b     = NTT(cP.b)
 *   c[lvl][k1].a[k2]  = sum_l' D_l' . s2[l'].a[k2] + NTT(cP.b)
 *   c[lvl][k1].b      = sum_l' D_l' . s2[l'].b                       (all mod q).
 */
/* blindRotateLazyPipeAltNtt (yatfhe/src/blind_rotate.cpp:995-1135), or with no_first
 * blindRotateLazyPipeAltNoFirstNtt (:1137-1267): the accumulator starts as X^-b (0, v) and
 * every key index, the first one included, takes the ordinary chain (rotate, decompose,
 * scheme switch, in-place external product). */
static int blind_rotate_lazy(const po_ctx* c, ep_scratch* s, const int32_t* scaled, const int64_t* v, int64_t* acc,
                             int no_first) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, k1 = k + 1, L = c->L, Ls = c->p.l, T = c->T;
    const int rb = c->p.radix_bits;
    const uint64_t q = c->q;
    const nq_barrett* br = &c->plan.br;
    const size_t row = (size_t)k1 * N, lvlWords = (size_t)k1 * row;
    if (!c->lazy_cprime || !c->wwl_s2 || n < (no_first ? 1 : 2) || L > 64 || Ls > 64) return -1;
    uint64_t* rows = (uint64_t*)malloc(sizeof(uint64_t) * L * lvlWords);  /* [lvl][r][o][N] */
    uint64_t* recomp = (uint64_t*)malloc(sizeof(uint64_t) * Ls * N);      /* NTT(2^(T-(l'+1) radix)) */
    uint64_t* gdv = (uint64_t*)malloc(sizeof(uint64_t) * L * N);
    uint64_t* hat = (uint64_t*)malloc(sizeof(uint64_t) * row);
    uint64_t* t1 = (uint64_t*)malloc(sizeof(uint64_t) * N);
    uint64_t* bh = (uint64_t*)malloc(sizeof(uint64_t) * N);
    int64_t* hold = (int64_t*)malloc(sizeof(int64_t) * row);
    int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * row);
    int64_t* dig = (int64_t*)malloc(sizeof(int64_t) * (size_t)(L > Ls ? L : Ls) * N);
    int64_t dg[64];
    int rc = -1;
    if (!rows || !recomp || !gdv || !hat || !t1 || !bh || !hold || !tmp || !dig) goto out;

    for (int gl = 0; gl < Ls; gl++) {
        memset(tmp, 0, sizeof(int64_t) * N);
        tmp[0] = sext((int64_t)1 << (T - (gl + 1) * rb), T);
        ntt_from_torus(c, recomp + (size_t)gl * N, tmp);
    }
    for (int j = 0; j < N; j++) {
        zero_mean_digits((uint64_t)v[j], L, rb, T, dg);
        for (int l = 0; l < L; l++) dig[(size_t)l * N + j] = dg[l];
    }
    for (int l = 0; l < L; l++) ntt_from_torus(c, gdv + (size_t)l * N, dig + (size_t)l * N);

    if (no_first) {
        /* the accumulator init of blindRotateLazyPipeAltNoFirstNtt (:1205-1210): X^-b (0, v) */
        memset(tmp, 0, sizeof(int64_t) * row);
        for (int j = 0; j < N; j++) tmp[(size_t)k * N + j] = v[j];
        for (int o = 0; o < k1; o++) rotate_poly(c, acc + (size_t)o * N, tmp + (size_t)o * N, -scaled[n], 0);
        goto chain;
    }
    /* first component */
    memset(hat, 0, sizeof(uint64_t) * row);
    for (int lvl = 0; lvl < L; lvl++) {
        const int64_t* cp = c->lazy_cprime + (size_t)lvl * row;  /* i = 0 */
        for (int o = 0; o < k1; o++) {
            ntt_from_torus(c, t1, cp + (size_t)o * N);
            uint64_t* h = hat + (size_t)o * N;
            for (int j = 0; j < N; j++) h[j] = addmod(h[j], nq_mulmod(br, gdv[(size_t)lvl * N + j], t1[j]), q);
        }
    }
    for (int o = 0; o < k1; o++) intt_to_torus(c, hold + (size_t)o * N, hat + (size_t)o * N);
    for (int o = 0; o < k1; o++) rotate_poly(c, tmp + (size_t)o * N, hold + (size_t)o * N, scaled[0], 1);
    for (int j = 0; j < N; j++) tmp[(size_t)k * N + j] = sext(tmp[(size_t)k * N + j] + v[j], T);
    for (int o = 0; o < k1; o++) rotate_poly(c, acc + (size_t)o * N, tmp + (size_t)o * N, -scaled[n], 0);

chain:
    for (int i = no_first ? 0 : 1; i < n; i++) {
        const int a = scaled[i];
        if (a == 0) continue;
        for (int lvl = 0; lvl < L; lvl++) {
            const int64_t* cp = c->lazy_cprime + ((size_t)i * L + lvl) * row;
            uint64_t* R = rows + (size_t)lvl * lvlWords;  /* R[r][o]: r < k c[lvl][r], r = k cPrime[lvl] */
            for (int o = 0; o < k1; o++) rotate_poly(c, hold + (size_t)o * N, cp + (size_t)o * N, a, 1);
            hold[(size_t)k * N] = sext(hold[(size_t)k * N] + ((int64_t)1 << (T - (lvl + 1) * rb)), T);
            memset(R, 0, sizeof(uint64_t) * lvlWords);
            ntt_from_torus(c, bh, hold + (size_t)k * N);
            for (int r = 0; r < k; r++) {
                for (int j = 0; j < N; j++) {
                    zero_mean_digits((uint64_t)hold[(size_t)r * N + j], Ls, rb, T, dg);
                    for (int gl = 0; gl < Ls; gl++) dig[(size_t)gl * N + j] = dg[gl];
                }
                for (int gl = 0; gl < Ls; gl++) {
                    ntt_from_torus(c, t1, dig + (size_t)gl * N);
                    const uint64_t* s2 = c->wwl_s2 + (size_t)gl * row;
                    uint64_t* cpa = R + (size_t)k * row + (size_t)r * N;
                    for (int j = 0; j < N; j++)
                        cpa[j] = addmod(cpa[j], nq_mulmod(br, t1[j], recomp[(size_t)gl * N + j]), q);
                    for (int o = 0; o < k1; o++) {
                        uint64_t* cr = R + (size_t)r * row + (size_t)o * N;
                        for (int j = 0; j < N; j++) cr[j] = addmod(cr[j], nq_mulmod(br, t1[j], s2[(size_t)o * N + j]), q);
                    }
                }
                for (int k2 = 0; k2 < k; k2++) {
                    uint64_t* cr = R + (size_t)r * row + (size_t)k2 * N;
                    for (int j = 0; j < N; j++) cr[j] = addmod(cr[j], bh[j], q);
                }
            }
            memcpy(R + (size_t)k * row + (size_t)k * N, bh, sizeof(uint64_t) * N);
        }
        external_product(c, s, rows, acc, acc);
    }
    rc = 0;
out:
    free(rows); free(recomp); free(gdv); free(hat); free(t1); free(bh); free(hold); free(tmp); free(dig);
    return rc;
}

int po_blind_rotate_lazy(po_ctx* c, const int32_t* in, const int64_t* v, int64_t* acc_out) {
    ep_scratch s;
    int32_t* scaled = (int32_t*)malloc(sizeof(int32_t) * (c->p.n + 1));
    if (ep_alloc(c, &s) || !scaled) {
        ep_free(&s);
        free(scaled);
        return fail(c, "po_blind_rotate_lazy: out of memory");
    }
    po_modswitch(c, in, scaled);
    const int rc = blind_rotate_lazy(c, &s, scaled, v, acc_out, 0);
    ep_free(&s);
    free(scaled);
    return rc ? fail(c, "po_blind_rotate_lazy: no lazy key, or n < 2") : 0;
}

/* functionalBootstrappingMPNtt's composition (yatfhe/src/bootstrapping.cpp:71-80) with
 * blindRotateLazyPipeAltNtt in place of blindRotateMP21Ntt. */
int po_pbs_lazy(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads) {
    if (!c->lazy_cprime || !c->wwl_s2) return fail(c, "po_pbs_lazy: no lazy key");
    return pbs_run(c, in, count, v, out, threads, 1);
}

/* The same two with blindRotateLazyPipeAltNoFirstNtt (yatfhe/src/blind_rotate.cpp:1137-1267). */
int po_blind_rotate_lazy_no_first(po_ctx* c, const int32_t* in, const int64_t* v, int64_t* acc_out) {
    ep_scratch s;
    int32_t* scaled = (int32_t*)malloc(sizeof(int32_t) * (c->p.n + 1));
    if (ep_alloc(c, &s) || !scaled) {
        ep_free(&s);
        free(scaled);
        return fail(c, "po_blind_rotate_lazy_no_first: out of memory");
    }
    po_modswitch(c, in, scaled);
    const int rc = blind_rotate_lazy(c, &s, scaled, v, acc_out, 1);
    ep_free(&s);
    free(scaled);
    return rc ? fail(c, "po_blind_rotate_lazy_no_first: no lazy key") : 0;
}

int po_pbs_lazy_no_first(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads) {
    if (!c->lazy_cprime || !c->wwl_s2) return fail(c, "po_pbs_lazy_no_first: no lazy key");
    return pbs_run(c, in, count, v, out, threads, 3);
}

/* ------------------------------------------------------------------ group keys */

/*
 * The key family of blindRotateNtt (BootstrappingKey, yatfhe/include/yatfhe/bootstrapping.h:16-45):
 * TrgswDft rows [lvl < l][row <= k] (trgsw.h:121-135), one TRGSW per LWE coefficient for
 * group 1, else 2^g per group of g coefficients, TRGSW k2 of a group encrypting
 * [combined == k2] with combined = sum_i2 s_(i+i2) 2^(g-1-i2) (genBootstrappingKeyGroup,
 * yatfhe/src/bootstrapping.cpp:16-38).
 */
static size_t grp_keys(const po_ctx* c, int g) {
    return g == 1 ? (size_t)c->p.n : (size_t)(c->p.n / g) << g;
}
static size_t grp_trgsw_words(const po_ctx* c) {
    const size_t k1 = (size_t)c->p.k + 1;
    return (size_t)c->p.l * k1 * k1 * c->p.N;
}

static int grp_alloc(po_ctx* c, int g) {
    if (g < 1 || g > 3 || c->p.n % g) return -1;
    free(c->grp_bsk);
    c->grp_bsk = (uint64_t*)calloc(grp_keys(c, g) * grp_trgsw_words(c), sizeof(uint64_t));
    c->grp = c->grp_bsk ? g : 0;
    return c->grp_bsk ? 0 : -1;
}

/* encryptTrgswNtt (yatfhe/src/trgsw.cpp:281-284): encZeroTrgswNtt (:185-191), one
 * symEncTrlweSingleSampleNtt of 0 per (lvl, row) (yatfhe/src/trlwe.cpp:88-91: noise b, uniform
 * masks, NTT-domain b + a . s), then addIntegerToTrgswNtt (:227-246): mu 2^(T-(lvl+1) radix)
 * added to coefficient 0 of a[row] (row < k) or of b (row k) in the torus domain, that
 * polynomial transformed again (its b comes back from applyIntt, reduced to T bits). */
static void enc_trgsw_group(po_ctx* c, uint64_t* out, int mu, int64_t* tmpT, int64_t* zero) {
    const int N = c->p.N, k = c->p.k, l = c->p.l, T = c->T;
    const size_t row = (size_t)(k + 1) * N;
    for (int lvl = 0; lvl < l; lvl++)
        for (int r = 0; r <= k; r++) enc_trlwe_coef_ntt(c, out + ((size_t)lvl * (k + 1) + r) * row, zero, tmpT);
    uint64_t* scratch = (uint64_t*)tmpT + 0;  /* reuses tmpT's storage as transform scratch */
    for (int lvl = 0; lvl < l; lvl++) {
        const int64_t g = sext((int64_t)mu << (T - (lvl + 1) * c->p.radix_bits), T);
        for (int r = 0; r <= k; r++) {
            uint64_t* poly = out + ((size_t)lvl * (k + 1) + r) * row + (size_t)r * N;  /* a[r], or b for r = k */
            memcpy(scratch, poly, sizeof(uint64_t) * N);
            intt_to_torus(c, zero, scratch);
            zero[0] = sext(zero[0] + g, T);
            ntt_from_torus(c, poly, zero);
            memset(zero, 0, sizeof(int64_t) * N);
        }
    }
}

int po_keygen_group(po_ctx* c, uint64_t seed, int group) {
    const int n = c->p.n, N = c->p.N;
    if (grp_alloc(c, group)) return fail(c, "po_keygen_group: group must be 1, 2 or 3 and divide n");
    int64_t* tmpT = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    int64_t* zero = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    if (!tmpT || !zero) {
        free(tmpT); free(zero);
        return fail(c, "po_keygen_group: out of memory");
    }
    keygen_secrets(c, seed, tmpT);
    const size_t tw = grp_trgsw_words(c);
    if (group == 1) {
        for (int i = 0; i < n; i++) enc_trgsw_group(c, c->grp_bsk + (size_t)i * tw, c->lwe_s[i], tmpT, zero);
    } else {
        size_t j = 0;
        for (int i = 0; i < n; i += group) {
            int combined = 0;
            for (int i2 = 0; i2 < group; i2++) combined |= c->lwe_s[i + i2] << (group - 1 - i2);
            for (int k2 = 0; k2 < (1 << group); k2++, j++)
                enc_trgsw_group(c, c->grp_bsk + j * tw, combined == k2, tmpT, zero);
        }
    }
    free(tmpT);
    free(zero);
    keygen_ksk(c);
    return 0;
}

int po_get_group(po_ctx* c, uint64_t* out) {
    if (!c->grp_bsk) return fail(c, "po_get_group: no group key");
    memcpy(out, c->grp_bsk, sizeof(uint64_t) * grp_keys(c, c->grp) * grp_trgsw_words(c));
    return 0;
}

int po_set_group(po_ctx* c, const uint64_t* words, int group) {
    if (grp_alloc(c, group)) return fail(c, "po_set_group: group must be 1, 2 or 3 and divide n");
    memcpy(c->grp_bsk, words, sizeof(uint64_t) * grp_keys(c, group) * grp_trgsw_words(c));
    return 0;
}

/* externalProductTrgswNtt (yatfhe/src/trgsw.cpp:550-576): every input polynomial decomposed
 * into l digit polynomials (gadgetDecomposeTrlwe), the first `level` of them transformed and
 * multiplied with key rows [lvl][col][col2], summed mod q, inverse transform.  key =
 * [l][k+1][k+1][N]; in/out = [a_0..a_{k-1}, b], may alias. */
static void ep_group(const po_ctx* c, const uint64_t* key, const int64_t* in, int64_t* out, int level,
                     int64_t* digits, uint64_t* dntt, uint64_t* acc) {
    const int N = c->p.N, k1 = c->p.k + 1, l = c->p.l;
    const uint64_t q = c->q;
    const size_t row = (size_t)k1 * N;
    int64_t dg[64];
    memset(acc, 0, sizeof(uint64_t) * row);
    for (int col = 0; col < k1; col++) {
        for (int j = 0; j < N; j++) {
            zero_mean_digits((uint64_t)in[(size_t)col * N + j], l, c->p.radix_bits, c->T, dg);
            for (int lv = 0; lv < level; lv++) digits[(size_t)lv * N + j] = dg[lv];
        }
        for (int lv = 0; lv < level; lv++) {
            ntt_from_torus(c, dntt, digits + (size_t)lv * N);
            const uint64_t* kr = key + ((size_t)lv * k1 + col) * row;
            for (int o = 0; o < k1; o++)
                for (int j = 0; j < N; j++)
                    acc[(size_t)o * N + j] = addmod(acc[(size_t)o * N + j],
                                                    nq_mulmod(&c->plan.br, dntt[j], kr[(size_t)o * N + j]), q);
        }
    }
    for (int o = 0; o < k1; o++) intt_to_torus(c, out + (size_t)o * N, acc + (size_t)o * N);
}

/*
 * blindRotateNtt (yatfhe/src/blind_rotate.cpp:549-560) on the group key, after
 * genNoiselessTrlweSample:
 *   group 1 (blindRotateNormalNtt, :202-212): for a_i != 0, acc += EP(K_i, X^(a_i) acc - acc)
 *     (controlMuxNtt, yatfhe/src/cmux.cpp:16-21);
 *   group g > 1 (blindRotateGroup2Ntt :264-324, blindRotateGroup3Ntt :398-488): per group of g
 *     coefficients acc = EP(sum_k2 rotateTrgswNtt(K_k2, r_k2), acc), r_k2 the sum of the a's whose
 *     bit is set in k2 (k2 = 1 is the last coefficient of the group); rotateTrgswNtt multiplies
 *     each polynomial by NTT(+-X^r') (rotateNttPolynomial, yatfhe/src/polynomial.cpp:405-412,
 *     with validateRotator's r' and sign; unchanged when r = 0 mod 2N).
 * The external products use lApprox of the key's l levels.
 */
static int blind_rotate_group(const po_ctx* c, const int32_t* scaled, const int64_t* v, int64_t* acc) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, k1 = k + 1, l = c->p.l, L = c->L, g = c->grp;
    const uint64_t q = c->q;
    const size_t row = (size_t)k1 * N, tw = grp_trgsw_words(c), lvw = (size_t)k1 * row;
    if (!c->grp_bsk || g < 1 || L > l || l > 64) return -1;
    int64_t* digits = (int64_t*)malloc(sizeof(int64_t) * (size_t)L * N);
    uint64_t* dntt = (uint64_t*)malloc(sizeof(uint64_t) * N);
    uint64_t* hat = (uint64_t*)malloc(sizeof(uint64_t) * row);
    int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * row);
    int64_t* mono = (int64_t*)malloc(sizeof(int64_t) * N);
    uint64_t* rot = (uint64_t*)malloc(sizeof(uint64_t) * N * 8);
    uint64_t* comb = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)L * lvw);
    int rc = -1;
    if (!digits || !dntt || !hat || !tmp || !mono || !rot || !comb) goto out;
    memset(acc, 0, sizeof(int64_t) * (size_t)k * N);
    rotate_poly(c, acc + (size_t)k * N, v, -scaled[n], 0);
    if (g == 1) {
        for (int i = 0; i < n; i++) {
            const int a = scaled[i];
            if (a == 0) continue;
            for (int r = 0; r < k1; r++) rotate_poly(c, tmp + (size_t)r * N, acc + (size_t)r * N, a, 1);
            ep_group(c, c->grp_bsk + (size_t)i * tw, tmp, tmp, L, digits, dntt, hat);
            for (size_t j = 0; j < row; j++) acc[j] = sext(acc[j] + tmp[j], c->T);
        }
    } else {
        for (int i = 0; i < n; i += g) {
            const uint64_t* keys = c->grp_bsk + (size_t)(i / g) * ((size_t)1 << g) * tw;
            for (int k2 = 0; k2 < (1 << g); k2++) {
                int r = 0;
                for (int i2 = 0; i2 < g; i2++)
                    if ((k2 >> (g - 1 - i2)) & 1) r += scaled[i + i2];
                int t = r % (2 * N);
                if (t < 0) t += 2 * N;
                memset(mono, 0, sizeof(int64_t) * N);
                if (t < N) mono[t] = 1; else mono[t - N] = -1;
                ntt_from_torus(c, rot + (size_t)k2 * N, mono);
            }
            for (int lv = 0; lv < L; lv++)
                for (size_t x = 0; x < lvw; x++) {
                    const size_t j = x % N;
                    uint64_t s = 0;
                    for (int k2 = 0; k2 < (1 << g); k2++) {
                        const uint64_t w = keys[(size_t)k2 * tw + (size_t)lv * lvw + x];
                        s = addmod(s, k2 == 0 ? w : nq_mulmod(&c->plan.br, w, rot[(size_t)k2 * N + j]), q);
                    }
                    comb[(size_t)lv * lvw + x] = s;
                }
            /* comb has the key's [lvl][col][col2] layout for its first L levels */
            ep_group(c, comb, acc, acc, L, digits, dntt, hat);
        }
    }
    rc = 0;
out:
    free(digits); free(dntt); free(hat); free(tmp); free(mono); free(rot); free(comb);
    return rc;
}

int po_blind_rotate_group(po_ctx* c, const int32_t* in, const int64_t* v, int64_t* acc_out) {
    int32_t* scaled = (int32_t*)malloc(sizeof(int32_t) * (c->p.n + 1));
    if (!scaled) return fail(c, "po_blind_rotate_group: out of memory");
    po_modswitch(c, in, scaled);
    const int rc = blind_rotate_group(c, scaled, v, acc_out);
    free(scaled);
    return rc ? fail(c, "po_blind_rotate_group: no group key") : 0;
}

/* functionalBootstrappingNtt (yatfhe/src/bootstrapping.cpp:60-68) on the group key. */
int po_pbs_group(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads) {
    if (!c->grp_bsk) return fail(c, "po_pbs_group: no group key");
    return pbs_run(c, in, count, v, out, threads, 2);
}

/* ------------------------------------------------------------------ approximate CRT (ApproxCRT) */

/*
 * blindRotateApproxCRTNtt (yatfhe/src/blind_rotate.cpp:577-589) with the conversions the
 * reference's BLIND_ROT_APPROX_CRT_NTT test puts around it (google_tests/blindrot_test.cpp:
 * 633-636): decompTrlweMcrt, the rotation, trlweMcrtToCrt, recompTrlweCrt
 * (yatfhe/include/yatfhe/trlwe.h:333-440).  The torus is Q_CRT = 251 241 239 233; the
 * accumulator is kept as d = 4 residue samples (int8, centred mod q_d, the low primes
 * scaled by taoU); per step (controlMuxApproxCRTNtt, yatfhe/src/cmux.cpp:45-57):
 *   tmp_d = X^a acc_d - acc_d mod q_d (rotateInt8PolynomialMinusOne, polynomial.cpp:262-271);
 *   decompTrlweApproxCrt (yatfhe/src/crt.cpp:102-140): low = 233 tmp_2 + 239 tmp_3 (the
 *     qLow / ql weights), digit_l = intModP(tmp_l - low, q_l) for the two high primes;
 *   broadcastTrlweApproxCrt (crt.cpp:142-164): digit_l reduced mod q_d where |digit_l| > q_d / 2;
 *   externalProductTrgswApproxCrtNtt (yatfhe/src/trgsw.cpp:607-657): the negacyclic products
 *     with the key rows summed mod MOD = 2^24 - 2^14 + 1 (NttNative24), centred mod MOD, then
 *     centred mod q_d (applyIntt, yatfhe/src/ntt24.cpp:222-240);
 *   accumulateTrlweModP: acc_d = longModP(res_d + acc_d, q_d).
 * The products go through this file's own negacyclic NTT mod MOD: any exact negacyclic
 * product mod MOD gives the same integers as the reference's NTT24.
 * bsk8: int8 [n][d][dh][k+1 rows][k+1 polys][N] (k = 1); in, out: torus values [2][N] (a, b);
 * rot: the rotation amounts [n]; mcrt (may be NULL): int8 [d][2][N] residues after the rotation.
 */
#define PO_CRT_D 4
#define PO_CRT_DH 2
#define PO_CRT_MOD 16760833u /* (1 << 24) - (1 << 14) + 1 */
static const int po_crt_q[PO_CRT_D] = {251, 241, 239, 233};

static int crt_mod_p(int64_t a, int64_t p) { return (int)int_mod_p(a, p); }

static uint32_t crt_pow(uint64_t b, uint64_t e) {
    uint64_t r = 1;
    b %= PO_CRT_MOD;
    while (e) {
        if (e & 1) r = r * b % PO_CRT_MOD;
        b = b * b % PO_CRT_MOD;
        e >>= 1;
    }
    return (uint32_t)r;
}

typedef struct {
    int N, logN;
    uint32_t* w;     /* psi^brv(k), k < N */
    uint32_t* wi;    /* psi^-brv(k) */
    uint32_t ninv;
} crt_ntt;

static int crt_brv(int x, int bits) {
    int r = 0;
    for (int i = 0; i < bits; i++) r |= ((x >> i) & 1) << (bits - 1 - i);
    return r;
}

static int crt_ntt_init(crt_ntt* t, int N) {
    t->N = N;
    t->logN = 0;
    while ((1 << t->logN) < N) t->logN++;
    t->w = (uint32_t*)malloc(sizeof(uint32_t) * N);
    t->wi = (uint32_t*)malloc(sizeof(uint32_t) * N);
    if (!t->w || !t->wi) return -1;
    /* 7 generates the multiplicative group mod MOD (NttNative24::PRIM_ROOT) */
    const uint32_t psi = crt_pow(7, (PO_CRT_MOD - 1) / (2 * (uint64_t)N));
    const uint32_t psi_inv = crt_pow(psi, PO_CRT_MOD - 2);
    for (int k = 0; k < N; k++) {
        t->w[k] = crt_pow(psi, (uint64_t)crt_brv(k, t->logN));
        t->wi[k] = crt_pow(psi_inv, (uint64_t)crt_brv(k, t->logN));
    }
    t->ninv = crt_pow((uint64_t)N, PO_CRT_MOD - 2);
    return 0;
}

static void crt_ntt_free(crt_ntt* t) {
    free(t->w);
    free(t->wi);
}

/* negacyclic forward (Cooley-Tukey, bit-reversed out) and inverse (Gentleman-Sande) mod MOD */
static void crt_fwd(const crt_ntt* t, uint32_t* a) {
    const int N = t->N;
    for (int m = 1, span = N / 2; m < N; m <<= 1, span >>= 1)
        for (int g = 0; g < m; g++)
            for (int j = 2 * g * span; j < 2 * g * span + span; j++) {
                const uint32_t u = a[j], v = (uint32_t)((uint64_t)a[j + span] * t->w[m + g] % PO_CRT_MOD);
                a[j] = u + v >= PO_CRT_MOD ? u + v - PO_CRT_MOD : u + v;
                a[j + span] = u >= v ? u - v : u + PO_CRT_MOD - v;
            }
}

static void crt_inv(const crt_ntt* t, uint32_t* a) {
    const int N = t->N;
    for (int m = N / 2, span = 1; m >= 1; m >>= 1, span <<= 1)
        for (int g = 0; g < m; g++)
            for (int j = 2 * g * span; j < 2 * g * span + span; j++) {
                const uint32_t u = a[j], v = a[j + span];
                a[j] = u + v >= PO_CRT_MOD ? u + v - PO_CRT_MOD : u + v;
                a[j + span] = (uint32_t)((uint64_t)(u >= v ? u - v : u + PO_CRT_MOD - v) * t->wi[m + g] % PO_CRT_MOD);
            }
    for (int j = 0; j < N; j++) a[j] = (uint32_t)((uint64_t)a[j] * t->ninv % PO_CRT_MOD);
}

static uint32_t crt_lift(int v) { return (uint32_t)((v % (int)PO_CRT_MOD + (int)PO_CRT_MOD) % (int)PO_CRT_MOD); }

/* The constants of initYatfhe (yatfhe/src/initializer.cpp:31-83): taoU / taoUInv of the low
 * primes and the CRT weights z_d = (Q/q_d) ((Q/q_d)^-1 mod q_d). */
static int64_t crt_inv_small(int64_t a, int64_t m) {
    a %= m;
    if (a < 0) a += m;
    for (int64_t x = 1; x < m; x++)
        if (a * x % m == 1) return x;
    return 0;
}

int po_crt_blind_rotate(int n, int N, const int8_t* bsk8, const int64_t* in, const int32_t* rot, int64_t* out,
                        int8_t* mcrt) {
    if (n < 1 || (N & (N - 1)) || N < 2 || N > 4096 || !bsk8 || !in || !rot || !out) return -1;
    const int64_t qLow = (int64_t)po_crt_q[2] * po_crt_q[3];
    const int64_t qCRT = (int64_t)po_crt_q[0] * po_crt_q[1] * qLow;
    int64_t taoU[PO_CRT_D] = {1, 1, 1, 1}, taoUInv[PO_CRT_D] = {1, 1, 1, 1}, z[PO_CRT_D];
    for (int u = 0; u < 2; u++) {
        const int64_t ql = po_crt_q[PO_CRT_DH + u];
        taoU[PO_CRT_DH + u] = crt_inv_small(qLow / ql, ql);
        taoUInv[PO_CRT_DH + u] = int_mod_p(qLow / ql, ql);
    }
    for (int d = 0; d < PO_CRT_D; d++) {
        const int64_t qt = qCRT / po_crt_q[d];
        z[d] = qt * crt_inv_small(qt, po_crt_q[d]);
    }
    const int64_t lowW[2] = {qLow / po_crt_q[2], qLow / po_crt_q[3]};
    crt_ntt t;
    if (crt_ntt_init(&t, N)) return -1;
    const size_t polys = (size_t)n * PO_CRT_D * PO_CRT_DH * 2 * 2;
    uint32_t* key = (uint32_t*)malloc(sizeof(uint32_t) * polys * N);
    int* acc = (int*)malloc(sizeof(int) * PO_CRT_D * 2 * N);
    int* nxt = (int*)malloc(sizeof(int) * PO_CRT_D * 2 * N);
    int* dig = (int*)malloc(sizeof(int) * PO_CRT_DH * 2 * N);
    uint32_t* x = (uint32_t*)malloc(sizeof(uint32_t) * N);
    uint32_t* sum = (uint32_t*)malloc(sizeof(uint32_t) * 2 * N);
    if (!key || !acc || !nxt || !dig || !x || !sum) {
        free(key); free(acc); free(nxt); free(dig); free(x); free(sum);
        crt_ntt_free(&t);
        return -1;
    }
    for (size_t pi = 0; pi < polys; pi++) {
        uint32_t* kp = key + pi * N;
        for (int j = 0; j < N; j++) kp[j] = crt_lift(bsk8[pi * N + j]);
        crt_fwd(&t, kp);
    }
    /* decompTrlweMcrt */
    for (int d = 0; d < PO_CRT_D; d++)
        for (int r = 0; r < 2; r++)
            for (int j = 0; j < N; j++) acc[(d * 2 + r) * N + j] = crt_mod_p(taoU[d] * in[r * N + j], po_crt_q[d]);
    for (int i = 0; i < n; i++) {
        if (rot[i] == 0) continue;
        int a = rot[i] % (2 * N);
        if (a < 0) a += 2 * N;
        const int wrapSign = a < N ? 1 : -1;
        if (a >= N) a -= N;
        /* rotate minus one, decompose, per coefficient */
        for (int r = 0; r < 2; r++)
            for (int j = 0; j < N; j++) {
                int tmp[PO_CRT_D];
                for (int d = 0; d < PO_CRT_D; d++) {
                    const int* A = acc + (d * 2 + r) * N;
                    const int v = (j < a ? -A[j - a + N] : A[j - a]) * wrapSign;
                    tmp[d] = crt_mod_p(v - A[j], po_crt_q[d]);
                }
                const int64_t low = lowW[0] * tmp[2] + lowW[1] * tmp[3];
                for (int l = 0; l < PO_CRT_DH; l++) dig[(l * 2 + r) * N + j] = crt_mod_p(tmp[l] - low, po_crt_q[l]);
            }
        for (int d = 0; d < PO_CRT_D; d++) {
            const int qd = po_crt_q[d], qdHalf = qd / 2;
            memset(sum, 0, sizeof(uint32_t) * 2 * N);
            for (int l = 0; l < PO_CRT_DH; l++)
                for (int r = 0; r < 2; r++) {
                    for (int j = 0; j < N; j++) {
                        const int v = dig[(l * 2 + r) * N + j];
                        x[j] = crt_lift(v > qdHalf || v < -qdHalf ? crt_mod_p(v, qd) : v);
                    }
                    crt_fwd(&t, x);
                    const uint32_t* kr = key + ((((size_t)i * PO_CRT_D + d) * PO_CRT_DH + l) * 2 + r) * 2 * N;
                    for (int c = 0; c < 2; c++)
                        for (int j = 0; j < N; j++)
                            sum[c * N + j] = (uint32_t)((sum[c * N + j] + (uint64_t)x[j] * kr[c * N + j]) % PO_CRT_MOD);
                }
            for (int c = 0; c < 2; c++) {
                crt_inv(&t, sum + c * N);
                for (int j = 0; j < N; j++) {
                    uint32_t v = sum[c * N + j];
                    const int centred = v >= (PO_CRT_MOD + 1) / 2 ? (int)v - (int)PO_CRT_MOD : (int)v;
                    const int res = crt_mod_p(centred, qd);
                    nxt[(d * 2 + c) * N + j] = crt_mod_p((int64_t)res + acc[(d * 2 + c) * N + j], qd);
                }
            }
        }
        int* sw = acc;
        acc = nxt;
        nxt = sw;
    }
    if (mcrt)
        for (size_t e = 0; e < (size_t)PO_CRT_D * 2 * N; e++) mcrt[e] = (int8_t)acc[e];
    /* trlweMcrtToCrt, recompTrlweCrt */
    for (int r = 0; r < 2; r++)
        for (int j = 0; j < N; j++) {
            int64_t s = 0;
            for (int d = 0; d < PO_CRT_D; d++) {
                int v = acc[(d * 2 + r) * N + j];
                if (d >= PO_CRT_DH) v = crt_mod_p(taoUInv[d] * v, po_crt_q[d]);
                s += (int64_t)v * z[d];
            }
            out[r * N + j] = int_mod_p(s, qCRT);
        }
    free(key); free(acc); free(nxt); free(dig); free(x); free(sum);
    crt_ntt_free(&t);
    return 0;
}
