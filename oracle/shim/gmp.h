/*
 * gmp.h -- stand-in for the handful of GMP mpz_* calls made by the reference's
 * native-NTT table builders (yatfhe/src/ntt64.cpp:80-103,136-148,
 * yatfhe/src/ntt16.cpp:33-41).  TEST INFRASTRUCTURE ONLY: it lets the reference's
 * own sources compile into the oracle under oracle/_ref/ without libgmp headers.
 * Every value those call sites handle is below 2^64 (moduli up to 2^64 - 2^32 + 1),
 * so one unsigned 128-bit integer per mpz_t is enough.
 */
#ifndef YATFHE_ORACLE_GMP_SHIM_H
#define YATFHE_ORACLE_GMP_SHIM_H

#include <stdarg.h>
#include <stddef.h>
#include <stdint.h>

typedef struct {
    unsigned __int128 v;
} __mpz_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpz_struct* mpz_ptr;
typedef const __mpz_struct* mpz_srcptr;

static inline void mpz_init(mpz_ptr x) { x->v = 0; }
static inline void mpz_clear(mpz_ptr x) { x->v = 0; }

static inline void mpz_inits(mpz_ptr x, ...) {
    va_list ap;
    va_start(ap, x);
    while (x) {
        x->v = 0;
        x = va_arg(ap, mpz_ptr);
    }
    va_end(ap);
}

static inline void mpz_clears(mpz_ptr x, ...) {
    va_list ap;
    va_start(ap, x);
    while (x) {
        x->v = 0;
        x = va_arg(ap, mpz_ptr);
    }
    va_end(ap);
}

static inline void mpz_set_ui(mpz_ptr x, unsigned long v) { x->v = v; }
static inline unsigned long mpz_get_ui(mpz_srcptr x) { return (unsigned long)(uint64_t)x->v; }

static inline void mpz_mul(mpz_ptr r, mpz_srcptr a, mpz_srcptr b) { r->v = a->v * b->v; }

static inline void mpz_mod(mpz_ptr r, mpz_srcptr a, mpz_srcptr m) { r->v = a->v % m->v; }

static inline void mpz_powm(mpz_ptr r, mpz_srcptr base, mpz_srcptr e, mpz_srcptr m) {
    unsigned __int128 mod = m->v, b = base->v % mod, acc = 1 % mod;
    unsigned __int128 k = e->v;
    while (k) {
        if (k & 1) acc = (acc * b) % mod;
        b = (b * b) % mod;
        k >>= 1;
    }
    r->v = acc;
}

/* Returns non-zero and sets r = a^-1 mod m when the inverse exists. */
static inline int mpz_invert(mpz_ptr r, mpz_srcptr a, mpz_srcptr m) {
    __int128 t = 0, newt = 1;
    __int128 rr = (__int128)m->v, newr = (__int128)(a->v % m->v);
    while (newr != 0) {
        __int128 qq = rr / newr, tmp;
        tmp = t - qq * newt; t = newt; newt = tmp;
        tmp = rr - qq * newr; rr = newr; newr = tmp;
    }
    if (rr > 1) return 0;
    if (t < 0) t += (__int128)m->v;
    r->v = (unsigned __int128)t;
    return 1;
}

#endif /* YATFHE_ORACLE_GMP_SHIM_H */
