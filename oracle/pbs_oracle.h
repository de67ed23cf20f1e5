/*
 * pbs_oracle.h -- plain-C restatement of the reference's TFHE programmable bootstrap
 * path (GINX / MP21), used as the correctness oracle.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the CPU-baseline leg
 * of bench.py call it to check or time against; the shipped library never links it.
 *
 * Conventions: torus values are int64 sign-extended from the torus width T (32 or 56);
 * LWE ciphertexts are int32 words [a_0 .. a_{n-1}, b] (mod 2^32);
 * NTT-domain key words are uint64 residues mod qNtt in the convention of ntt_q.h.
 */
#ifndef YATFHE_ORACLE_PBS_ORACLE_H
#define YATFHE_ORACLE_PBS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n, N, k, radix_bits, l, l_approx, ks_radix_bits, ks_level, lwe_noise_b, rlwe_noise_b, torus_base;
    int torus_bits; /* 32 or 56 */
} po_params;

typedef struct po_ctx po_ctx;

po_ctx* po_create(const po_params* p);
void po_destroy(po_ctx* c);
const char* po_last_error(po_ctx* c);
uint64_t po_qntt(po_ctx* c);

int po_keygen(po_ctx* c, uint64_t seed);
int po_encrypt(po_ctx* c, const int64_t* mu, int count, int32_t* out);
int po_encrypt_samples(po_ctx* c, const int64_t* mu, int count, int32_t* out, int32_t* mask, int32_t* noise);
int po_encrypt_rlwe_ntt_samples(po_ctx* c, const int64_t* mu, int count, uint64_t* out, uint64_t* mask,
                                int32_t* noise);
int po_decrypt(po_ctx* c, const int32_t* in, int count, int base, int32_t* out);

int po_get_keys(po_ctx* c, int32_t* lwe_s, int32_t* rlwe_s);
int po_set_keys(po_ctx* c, const int32_t* lwe_s, const int32_t* rlwe_s);
int po_get_ksk(po_ctx* c, int32_t* out);
int po_set_ksk(po_ctx* c, const int32_t* in);
int po_get_bsk_ntt(po_ctx* c, uint64_t* out);
int po_set_bsk_ntt(po_ctx* c, const uint64_t* in);
int po_save_bsk_file(po_ctx* c, const char* path);
int po_load_bsk_file(po_ctx* c, const char* path);

int po_test_polynomial(po_ctx* c, int kind, int modP, int64_t* v);
int po_modswitch(po_ctx* c, const int32_t* in, int32_t* out);
int po_rotate(po_ctx* c, const int64_t* in, int a, int minus_one, int64_t* out);
int po_decompose(po_ctx* c, const int64_t* in, int levels, int64_t* out);
int po_decompose_ks(po_ctx* c, int64_t value, int64_t* out);
int po_ntt_forward(po_ctx* c, const int64_t* in, uint64_t* out);
int po_ntt_inverse(po_ctx* c, const uint64_t* in, int64_t* out);
int po_external_product(po_ctx* c, const int64_t* in, int i, int64_t* out);
int po_extract(po_ctx* c, const int64_t* acc, int32_t* out);
int po_keyswitch(po_ctx* c, const int32_t* in, int32_t* out);
int po_blind_rotate_trace(po_ctx* c, const int32_t* in, const int64_t* v, const int* checkpoints, int ncheck,
                          int64_t* acc_out, int64_t* acc_final);
int po_pbs(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads);

/* WWL+24 keys (half TRGSW rows cPrime [n][l_approx][k+1][N] + s2 [l][k+1][N], NTT domain):
 * po_wwl24_expand writes the GINX rows the WWL+24 blind rotation derives from them into the
 * context's BSK, after which po_pbs / po_blind_rotate_trace run the WWL+24 bootstrap. */
int po_keygen_wwl24(po_ctx* c, uint64_t seed);
int po_get_wwl24(po_ctx* c, uint64_t* cprime, uint64_t* s2);
int po_set_wwl24(po_ctx* c, const uint64_t* cprime, const uint64_t* s2);
int po_wwl24_expand(po_ctx* c);
int po_save_wwl24_file(po_ctx* c, const char* path);
int po_load_wwl24_file(po_ctx* c, const char* path);

/* Lazy ("OURS") keys of blindRotateLazyPipeAltNtt: half TRGSW rows in the coefficient domain
 * cprime [n][l_approx][k+1][N] (torus values) + the s2 key [l][k+1][N] (NTT domain). */
int po_keygen_lazy(po_ctx* c, uint64_t seed);
int po_get_lazy(po_ctx* c, int64_t* cprime, uint64_t* s2);
int po_set_lazy(po_ctx* c, const int64_t* cprime, const uint64_t* s2);
int po_save_lazy_file(po_ctx* c, const char* path);
int po_load_lazy_file(po_ctx* c, const char* path);
int po_blind_rotate_lazy(po_ctx* c, const int32_t* in, const int64_t* v, int64_t* acc_out);
int po_pbs_lazy(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads);
int po_blind_rotate_lazy_no_first(po_ctx* c, const int32_t* in, const int64_t* v, int64_t* acc_out);
int po_pbs_lazy_no_first(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads);

/* Group-g keys of blindRotateNtt (BootstrappingKey, TrgswDft rows [keys][l][k+1][k+1][N] in the
 * NTT domain; keys = n for g = 1, n / g * 2^g otherwise; g divides n). */
int po_keygen_group(po_ctx* c, uint64_t seed, int group);
int po_get_group(po_ctx* c, uint64_t* out);
int po_set_group(po_ctx* c, const uint64_t* words, int group);
int po_blind_rotate_group(po_ctx* c, const int32_t* in, const int64_t* v, int64_t* acc_out);
int po_pbs_group(po_ctx* c, const int32_t* in, int count, const int64_t* v, int32_t* out, int threads);

/* po_keygen that also writes out its random samples (see pbs_oracle.c). */
int po_keygen_samples(po_ctx* c, uint64_t seed, int32_t* lwe_s, int32_t* rlwe_s, int32_t* bsk_noise,
                      uint64_t* bsk_mask, int32_t* ksk_mask, int32_t* ksk_noise);

/* The approximate-CRT blind rotation blindRotateApproxCRTNtt with its input and output
 * conversions (see pbs_oracle.c): bsk8 int8 [n][4][2][2][2][N], in/out torus values mod Q_CRT
 * [2][N], rot [n]; mcrt (may be NULL) int8 [4][2][N].  Needs no context. */
int po_crt_blind_rotate(int n, int N, const int8_t* bsk8, const int64_t* in, const int32_t* rot, int64_t* out,
                        int8_t* mcrt);

#ifdef __cplusplus
}
#endif

#endif /* YATFHE_ORACLE_PBS_ORACLE_H */
