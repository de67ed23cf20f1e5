/*
 * yatfhe_gb300.h -- C ABI of the GB300 programmable-bootstrap library.
 *
 * A drop-in for the GINX/MP21 bootstrap path of the yatfhe reference library, whose
 * public interface is a set of C++ free functions (no FFI layer of its own).  Each entry
 * point below names the reference interface it replaces.  Paths are relative to the
 * reference project.
 *
 * Conventions
 *   - Plain pointers and sizes, int status codes (YG_OK == 0); the message of the last
 *     failure on the calling thread is returned by yg_last_error().
 *   - LWE ciphertexts: int32 words [a_0 .. a_{n-1}, b] modulo 2^32 (the reference's Tlwe,
 *     yatfhe/include/yatfhe/tlwe.h:13-22; under TORUS56 it stores the same values in int64).
 *   - Test polynomials (LUTs): N int64 torus coefficients, sign-extended from T bits
 *     (TorusPolynomial, yatfhe/include/yatfhe/polynomial.h:17-40).
 *   - Functions taking d_* pointers expect device memory and enqueue on `stream` (a
 *     cudaStream_t, NULL = legacy default stream); they do not synchronize.  Functions
 *     taking h_* pointers copy to and from host memory and return when the results are in
 *     the host buffers.
 *   - Results are bit-identical to the reference's functions on the same keys and inputs.
 */
#ifndef YATFHE_GB300_H
#define YATFHE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define YG_OK 0
#define YG_ERR_INVALID (-1)   /* bad argument or unsupported parameters (std::invalid_argument) */
#define YG_ERR_CUDA (-2)      /* a CUDA call failed */
#define YG_ERR_IO (-3)        /* file missing, short or malformed (std::runtime_error) */
#define YG_ERR_NOMEM (-4)     /* host or device allocation failed */
#define YG_ERR_STATE (-5)     /* object used in the wrong state (e.g. no KSK loaded) */

/* The fields of YatfheParameters (yatfhe/include/yatfhe/yatfhe_parameters.h:9-110) that
 * the bootstrap reads: l_approx is the gadget level count of the key and of the
 * decomposition; ks_level / ks_radix_bits the key-switching decomposition. */
typedef struct yg_params {
    int n;
    int N;
    int k;
    int radix_bits;
    int l_approx;
    int ks_radix_bits;
    int ks_level;
    int torus_bits; /* 32 or 56 */
} yg_params;

typedef struct yg_ctx yg_ctx;
typedef struct yg_key yg_key;

/* Message of the last failed call on this thread ("" if none). */
const char* yg_last_error(void);

/* Replaces initYatfhe (yatfhe/src/initializer.cpp:50-85) for one parameter set; unlike it,
 * any number of contexts (parameter sets) may live in one process. */
int yg_ctx_create(const yg_params* params, int device, yg_ctx** out);
void yg_ctx_destroy(yg_ctx* ctx);

/* Replaces deserializeBskMP (yatfhe/src/ya_serializer.cpp:287-303): reads a GINX key
 * written by serializeBskMP (:276-285) and makes it device-resident. */
int yg_key_load_bsk_file(yg_ctx* ctx, const char* path, yg_key** out);

/* Same, from the NTT-domain words of BootstrappingKeyMP::bskDft
 * (yatfhe/include/yatfhe/bootstrapping.h:47-114) laid out [n][l][k+1][k+1][N]:
 * row r < k is c[lvl][r], row k is cPrime[lvl]; poly p < k is a[p], poly k is b. */
int yg_key_upload_bsk_ntt(yg_ctx* ctx, const uint64_t* h_bsk_ntt, yg_key** out);

/* Attaches the key-switching key (TlweKeySwitchingKey::decomposedKsk,
 * yatfhe/include/yatfhe/keyswitching.h:14-31) as int32 words [k N][t][n + 1]. */
int yg_key_set_ksk(yg_key* key, const int32_t* h_ksk);

void yg_key_destroy(yg_key* key);
size_t yg_key_device_bytes(const yg_key* key);

/* functionalBootstrappingMPNtt (yatfhe/src/bootstrapping.cpp:71-80) on `count`
 * ciphertexts under one key: d_in, d_out are [count][n + 1], d_lut is [N]. */
int yg_pbs(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, int32_t* d_out, int count, const int64_t* d_lut,
           void* stream);

/* yg_pbs with host buffers: copies in, bootstraps, copies out, synchronizes `stream`. */
int yg_pbs_host(yg_ctx* ctx, const yg_key* key, const int32_t* h_in, int32_t* h_out, int count,
                const int64_t* h_lut, void* stream);

/* No counterpart in the reference.  yg_pbs for callers that cannot let the library
 * allocate device memory (their memory is owned by their own allocator or budget, or
 * they reserve everything at start-up): the intermediate ciphertexts live in a fixed
 * 16 MiB array compiled into the library, resident on every GPU that loads it until the
 * process exits, instead of a per-call allocation.  At most yg_pbs_noalloc_max_count(ctx)
 * ciphertexts per call (4092 at N = 1024, 2046 at N = 2048); more is rejected with
 * YG_ERR_INVALID.  The first call on a device looks up the array's device address, so make
 * it before any stream capture.  All calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller. */
int yg_pbs_noalloc(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, int32_t* d_out, int count,
                   const int64_t* d_lut, void* stream);
size_t yg_pbs_noalloc_max_count(const yg_ctx* ctx);

/* rescaleTlweToNewMod + genNoiselessTrlweSample + the first `steps` iterations of
 * blindRotateMP21Ntt (yatfhe/src/blind_rotate.cpp:1538-1565; steps = n is the whole
 * rotation).  d_acc receives [count][(k+1) N] int64 torus words, a then b. */
int yg_blind_rotate(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, const int64_t* d_lut, int64_t* d_acc,
                    int count, int steps, void* stream);

/* blindRotateMP21Ntt with the reference's own signature semantics
 * (yatfhe/include/yatfhe/blind_rotate.h:69): d_scaled is ScaledTlwe::a ([count][n], values
 * mod 2N in [-N, N)), d_acc ([count][(k+1) N] int64, a then b) is rotated in place. */
int yg_blind_rotate_acc(yg_ctx* ctx, const yg_key* key, const int32_t* d_scaled, int64_t* d_acc, int count,
                        void* stream);

/* A key object holding only a key-switching key (attach it with yg_key_set_ksk), for
 * switchKeyForTlwe callers that have no bootstrapping key. */
int yg_key_create_ksk_only(yg_ctx* ctx, yg_key** out);

/* The first half of functionalBootstrappingMPNtt (yatfhe/src/bootstrapping.cpp:75-78):
 * rescale, noiseless sample, blindRotateMP21Ntt, extractTlweFromTrlwe(., ., 0).
 * d_big receives [count][k N + 1] int32 words; yg_keyswitch finishes the bootstrap. */
int yg_blind_rotate_extract(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, const int64_t* d_lut,
                            int32_t* d_big, int count, void* stream);

/* switchKeyForTlwe (yatfhe/src/keyswitching.cpp:48-72): d_big is [count][k N + 1]
 * (extractTlweFromTrlwe output), d_out is [count][n + 1]. */
int yg_keyswitch(yg_ctx* ctx, const yg_key* key, const int32_t* d_big, int32_t* d_out, int count, void* stream);

/* Calibration, no reference counterpart: measured 32-bit multiply-add throughput of
 * `device` (operations per second), the denominator of the bootstrap's roofline. */
int yg_probe_int32_rate(int device, double* ops_per_second);

#ifdef __cplusplus
}
#endif

#endif /* YATFHE_GB300_H */
