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
 * decomposition; ks_level / ks_radix_bits the key-switching decomposition.  Supported:
 * torus_bits 32 or 56, N 1024 or 2048, k = 1, n <= 4096, radix_bits <= 15, l_approx <= 15,
 * l_approx * radix_bits <= torus_bits, ks_level <= 16, ks_radix_bits <= 7, and gadgets
 * whose exact products stay inside the three-prime RNS; yg_ctx_create rejects the rest
 * with YG_ERR_INVALID. */
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
 * row r < k is c[lvl][r], row k is cPrime[lvl]; poly p < k is a[p], poly k is b.  The
 * conversion to the device form (inverse transform mod q, split into the RNS channels,
 * each channel's forward transform) runs on the GPU; a word not reduced mod q is rejected
 * with YG_ERR_INVALID.  Synchronizes the device. */
int yg_key_upload_bsk_ntt(yg_ctx* ctx, const uint64_t* h_bsk_ntt, yg_key** out);

/* WWL+24 keys (BootstrappingKeyWWL24, yatfhe/include/yatfhe/bootstrapping.h:116-135): the
 * half TRGSW rows cPrime of every key index, [n][l_approx][k+1][N], and the s2 key s2Dft
 * with s2_levels (the reference's param.l) levels, [s2_levels][k+1][N], NTT-domain words
 * mod q (poly p < k is a[p], poly k is b).  The GPU derives,
 * once per key, the GINX rows blindRotateWWL24Ntt (yatfhe/src/blind_rotate.cpp:1383-1412)
 * rebuilds before every external product (switchTrlweToSecretEmbeddingNtt,
 * yatfhe/src/trgsw.cpp:861-905), so the key handle then runs every bootstrap and
 * blind-rotation entry point below with the WWL+24 results.  Requires s2_levels <= 8 and
 * s2_levels * radix_bits <= torus_bits; a word not reduced mod q is rejected with YG_ERR_INVALID.  Synchronizes the device. */
int yg_key_upload_wwl24_ntt(yg_ctx* ctx, const uint64_t* h_cprime, const uint64_t* h_s2, int s2_levels,
                            yg_key** out);

/* Key generation on the GPU from caller-drawn randomness: the arithmetic of
 * genBootstrappingKeyMP's per-index encryptTrgswMPNtt (yatfhe/src/bootstrapping.cpp:150-174,
 * yatfhe/src/trgsw.cpp:36-51) and of genTlweKeySwitchingKey (yatfhe/src/keyswitching.cpp:19-29),
 * with the random samples supplied by the caller (the library draws none):
 *   h_lwe_s [n], h_rlwe_s [k N]: the binary secrets;
 *   h_bsk_noise [n][l_approx][k+1][N] int32: the TUniform noise of each RLWE sample's b
 *       (row k of a level is cPrime, rows r < k are c[lvl][r]);
 *   h_bsk_mask [n][l_approx][k+1][k][N]: each sample's uniform NTT-domain masks (< q);
 *   h_ksk_mask [k N][ks_level][n] int32, h_ksk_noise [k N][ks_level] int32: the key-switching
 *       samples' masks and noise.
 * Drawn in the reference's order from its RNG these give the reference's keys bit for bit.
 * Makes a device key with BSK and KSK; h_bsk_words ([n][l_approx][k+1][k+1][N], the layout of
 * yg_key_upload_bsk_ntt) and h_ksk ([k N][ks_level][n+1]) receive the keys when not null.
 * Non-binary secrets and unreduced masks are rejected with YG_ERR_INVALID.  Synchronizes. */
int yg_keygen_from_samples(yg_ctx* ctx, const int32_t* h_lwe_s, const int32_t* h_rlwe_s, const int32_t* h_bsk_noise,
                           const uint64_t* h_bsk_mask, const int32_t* h_ksk_mask, const int32_t* h_ksk_noise,
                           uint64_t* h_bsk_words, int32_t* h_ksk, yg_key** out);

/* Key generation with the randomness drawn on the GPU: the secrets (genTlweKey /
 * genTrlweKey, yatfhe/src/tlwe.cpp:10-18, yatfhe/src/trlwe.cpp:70-81: uniform bits), the BSK
 * samples' TUniform(rlwe_noise_b) noise and uniform masks mod q (encryptTrgswMPNtt,
 * yatfhe/src/trgsw.cpp:36-51; genTUniformNoise, yatfhe/src/numeric.cpp:47-55) and the KSK
 * samples' uniform 32-bit masks and TUniform(lwe_noise_b) noise (genTlweKeySwitchingKey,
 * yatfhe/src/keyswitching.cpp:19-29), then the arithmetic of yg_keygen_from_samples on them.
 * The generator is ChaCha20 (RFC 8439) in counter mode keyed by `seed` (one key per array),
 * so the same seed gives the same key on any GPU; the values have the reference's
 * distributions, not its words (its RNG is one sequential stream).  h_lwe_s [n] and
 * h_rlwe_s [k N] receive the secrets when not null.  0 <= lwe_noise_b, rlwe_noise_b <= 30
 * (the noise is kept as int32).  Synchronizes. */
int yg_keygen(yg_ctx* ctx, uint64_t seed, int lwe_noise_b, int rlwe_noise_b, int32_t* h_lwe_s, int32_t* h_rlwe_s,
              yg_key** out);

/* The samples yg_keygen draws for `seed`, in the layouts of yg_keygen_from_samples: fed back
 * to it they give yg_keygen's key bit for bit.  Synchronizes. */
int yg_draw_keygen_samples(yg_ctx* ctx, uint64_t seed, int lwe_noise_b, int rlwe_noise_b, int32_t* h_lwe_s,
                           int32_t* h_rlwe_s, int32_t* h_bsk_noise, uint64_t* h_bsk_mask, int32_t* h_ksk_mask,
                           int32_t* h_ksk_noise);

/* symEncTlwe (yatfhe/src/tlwe.cpp:21-31) of `count` messages on the GPU, one warp per
 * ciphertext: d_out[i] = (a, sum_j a_j s_j + mu_i + e_i mod 2^32) with d_s [n] the binary LWE
 * secret, d_mu [count] the torus messages (taken mod 2^32), uniform 32-bit masks a and
 * TUniform(lwe_noise_b) noise e drawn by ChaCha20 from (seed, call): one (seed, call) pair
 * gives one set of ciphertexts, so a caller encrypting in several calls gives each its own
 * `call`.  d_out is [count][n + 1] int32.  Device pointers; asynchronous on `stream`. */
int yg_encrypt_lwe(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, int count, uint64_t seed, uint32_t call,
                   int lwe_noise_b, int32_t* d_out, void* stream);

/* As yg_encrypt_lwe with the samples given: d_mask [count][n] and d_noise [count] (the
 * reference's draws give the reference's ciphertexts bit for bit). */
int yg_encrypt_lwe_from_samples(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, const int32_t* d_mask,
                                const int32_t* d_noise, int count, int32_t* d_out, void* stream);

/* symEncTrlweMultiSampleSimple (yatfhe/src/trlwe.cpp:40-47,62-64; yatfhe/include/yatfhe/trlwe.h:518)
 * of `count` torus polynomials on the GPU: d_out[i] = (a, NTT(sext(mu_i + e_i)) + a . NTT(s)
 * mod q), NTT-domain words [count][k+1][N] (a_0 .. a_{k-1}, b) with masks a uniform mod q and
 * TUniform(rlwe_noise_b) noise e drawn by ChaCha20 from (seed, call).  d_s [k N] is the binary
 * RLWE secret, d_mu [count][N] the plaintext torus coefficients (int64, reduced to the torus
 * width).  Device pointers; asynchronous on `stream` (its scratch comes from the stream's
 * memory pool).  Requires k = 1. */
int yg_encrypt_rlwe_ntt(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, int count, uint64_t seed, uint32_t call,
                        int rlwe_noise_b, uint64_t* d_out, void* stream);

/* As yg_encrypt_rlwe_ntt with the samples given: d_mask [count][k][N] (words < q) and d_noise
 * [count][N].  Synchronizes `stream`; a mask word >= q gives YG_ERR_INVALID. */
int yg_encrypt_rlwe_ntt_from_samples(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, const uint64_t* d_mask,
                                     const int32_t* d_noise, int count, uint64_t* d_out, void* stream);

/* The approximate-CRT blind rotation (blindRotateApproxCRTNtt, yatfhe/src/blind_rotate.cpp:
 * 577-589) with the conversions the reference's BLIND_ROT_APPROX_CRT_NTT test puts around it
 * (decompTrlweMcrt, trlweMcrtToCrt, recompTrlweCrt; yatfhe/include/yatfhe/trlwe.h:333-440), on
 * the torus Q_CRT = 251 241 239 233 with k = 1.  Its key is separate from yg_ctx: the residue
 * rows of BootstrappingKeyCRT::bsk8 (yatfhe/include/yatfhe/bootstrapping.h:351-361),
 * h_bsk8 int8 [n][4 primes][2 levels][2 rows][2 polys (a, b)][N], each a residue centred mod
 * its prime (|v| <= 125, else YG_ERR_INVALID); the device keeps their transforms mod
 * 2^24 - 2^14 + 1 (NttNative24's field), 16 N bytes per key row.  N = 1024 or 2048.
 * Synchronizes the device. */
typedef struct yg_crt_key yg_crt_key;
int yg_crt_key_upload(int device, int n, int N, const int8_t* h_bsk8, yg_crt_key** out);

/* d_acc_in [count][2][N]: each ciphertext's starting TRLWE sample (a then b) as torus values
 * mod Q_CRT (int32, centred); d_rot [count][n]: the rotation amounts a_i (any integers; taken
 * mod 2N, a_i = 0 skipped as the reference skips it); d_acc_out [count][2][N] receives the
 * rotated sample.  Device pointers; asynchronous on `stream`. */
int yg_crt_blind_rotate(yg_crt_key* key, const int32_t* d_acc_in, const int32_t* d_rot, int count, int32_t* d_acc_out,
                        void* stream);
size_t yg_crt_key_device_bytes(const yg_crt_key* key);
void yg_crt_key_destroy(yg_crt_key* key);

/* Replaces deserializeBskWWL24 (yatfhe/src/ya_serializer.cpp:231-246): reads a file written
 * by serializeBskWWL24 (:220-229) and uploads it as above. */
int yg_key_load_wwl24_file(yg_ctx* ctx, const char* path, yg_key** out);

/* Lazy ("OURS") keys (BootstrappingKeyMPLazyPipeAlt, yatfhe/include/yatfhe/bootstrapping.h:284-307):
 * the half TRGSW rows bskPrime[i].cPrime of every key index in the coefficient domain,
 * [n][l_approx][k+1][N] torus values sign-extended to int64 (poly p < k is a[p], poly k is
 * b), and the s2 key s2Dft with s2_levels (the reference's param.l) levels,
 * [s2_levels][k+1][N] NTT-domain words mod q.  The device keeps the rows as they are, in the
 * torus word size (4 bytes at T = 32, a quarter of the GINX rows' bytes), and every
 * bootstrap rebuilds each CMux step's TRGSW from them as blindRotateLazyPipeAltNtt
 * (yatfhe/src/blind_rotate.cpp:995-1135) does.  Such a key runs yg_pbs, yg_pbs_host,
 * yg_blind_rotate (steps = n), yg_blind_rotate_extract, the batch plans (with other lazy keys
 * of the same s2 levels) and the serving loop (a lazy-key server) with the lazy blind
 * rotation; yg_pbs_noalloc and yg_blind_rotate_acc reject it with YG_ERR_INVALID.  Requires n >= 2, l_approx <= 8, radix_bits <= 15, s2_levels <= 8 and
 * s2_levels * radix_bits <= torus_bits; an unreduced s2 word or a row value that is not a
 * sign-extended torus value is rejected with YG_ERR_INVALID.  Synchronizes the device. */
int yg_key_upload_lazy(yg_ctx* ctx, const int64_t* h_cprime, const uint64_t* h_s2, int s2_levels, yg_key** out);

/* Group-g keys (BootstrappingKey, yatfhe/include/yatfhe/bootstrapping.h:16-45, made by
 * genBootstrappingKey with param.group = group, yatfhe/src/bootstrapping.cpp:16-38,98-104): the
 * NTT-domain TrgswDft words of every key, [keys][key_levels][k+1][k+1][N] (trlweDftSamples[lvl][row],
 * poly p < k is a[p], poly k is b; keys = n for group 1, n / group * 2^group otherwise),
 * key_levels the reference's param.l.  The key handle runs blindRotateNtt
 * (yatfhe/src/blind_rotate.cpp:549-560: blindRotateNormalNtt, blindRotateGroup2Ntt or
 * blindRotateGroup3Ntt) in yg_pbs (then functionalBootstrappingNtt,
 * yatfhe/src/bootstrapping.cpp:60-68), yg_pbs_host, yg_blind_rotate (steps = n) and
 * yg_blind_rotate_extract and yg_blind_rotate_acc; the other entry points refuse it like a lazy key.  Requires group
 * 1, 2 or 3 dividing n, l_approx <= key_levels <= 8, key_levels * radix_bits <= torus_bits;
 * an unreduced word is rejected with YG_ERR_INVALID.  Synchronizes the device. */
int yg_key_upload_group(yg_ctx* ctx, const uint64_t* h_words, int group, int key_levels, yg_key** out);

/* Replaces deserializeBskLazyPipeAlt (yatfhe/src/ya_serializer.cpp:462-481): reads a file
 * written by serializeBskLazyPipeAlt (:445-460) and uploads it as above. */
int yg_key_load_lazy_file(yg_ctx* ctx, const char* path, yg_key** out);

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
 * YG_ERR_INVALID.  A call with count 0 (buffers may be NULL) only sets the device up: it
 * looks up the array's device address, which is when the CUDA driver commits the array's 16 MiB
 * on that device (it loads the library's device variables lazily), and loads the two
 * kernels a call launches.  Make that call at start-up, before any stream capture and
 * before the caller stops allowing allocations; otherwise the first call with count > 0 on
 * a device does the set-up itself.  All calls share the array: calls that overlap on the
 * GPU race and must be serialised by the caller. */
int yg_pbs_noalloc(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, int32_t* d_out, int count,
                   const int64_t* d_lut, void* stream);
size_t yg_pbs_noalloc_max_count(const yg_ctx* ctx);

/* rescaleTlweToNewMod + genNoiselessTrlweSample + the first `steps` iterations of
 * blindRotateMP21Ntt (yatfhe/src/blind_rotate.cpp:1538-1565; steps = n is the whole
 * rotation).  d_acc receives [count][(k+1) N] int64 torus words, a then b.  With a lazy key:
 * rescaleTlweToNewMod + blindRotateLazyPipeAltNtt, steps = n only. */
int yg_blind_rotate(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, const int64_t* d_lut, int64_t* d_acc,
                    int count, int steps, void* stream);

/* blindRotateMP21Ntt with the reference's own signature semantics
 * (yatfhe/include/yatfhe/blind_rotate.h:69): d_scaled is ScaledTlwe::a ([count][n], values
 * mod 2N in [-N, N)), d_acc ([count][(k+1) N] int64, a then b) is rotated in place.  With a
 * group key: blindRotateNtt (blind_rotate.h:13) in place, the same way; lazy keys are
 * refused (their rotation builds the accumulator from the test polynomial). */
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

/* Batches under many keys (no reference counterpart: the reference bootstraps one
 * ciphertext per call).  A plan fixes, ahead of time, which key and which test
 * polynomial each of `count` ciphertexts uses and owns the device tables and the
 * intermediate buffer; yg_plan_run then only launches kernels (two), so it may be captured
 * in a CUDA graph and replayed.  h_key_ids / h_lut_ids are host arrays of `count` indices
 * into keys[] / d_luts[] (NULL: every ciphertext uses entry 0).  Ciphertexts that share a
 * key should be contiguous: the key switch streams one KSK per run of them.  All keys must
 * belong to `ctx`, carry a KSK and be of one family: GINX rows (WWL+24 keys included) or
 * lazy keys with the same s2 levels (then the lazy blind rotation runs, the launch shape
 * below does not apply); group keys are refused. */
typedef struct yg_plan yg_plan;
int yg_plan_create(yg_ctx* ctx, const yg_key* const* keys, int num_keys, const int32_t* h_key_ids,
                   const int64_t* const* d_luts, int num_luts, const int32_t* h_lut_ids, int count, yg_plan** out);
/* Work split of one ciphertext in the blind rotation.  YG_LAYOUT_CHANNEL: one team of
 * N/32 threads per RNS channel runs every NTT of a CMux step.  YG_LAYOUT_CHANNEL_ROW: two
 * teams per channel, one per accumulator row, each running half the forward transforms and
 * one inverse transform: twice the threads per ciphertext, about half the latency.
 * YG_LAYOUT_ROW_CLUSTER (T = 32, N = 1024, l_approx <= 4, per_cta 1): a cluster of two CTAs
 * per ciphertext, one per accumulator row, with one team per (channel, digit level), so the
 * levels' transforms run side by side (the grid is always two CTAs per ciphertext; a
 * persistent grid does not apply).  YG_LAYOUT_CHANNEL_CLUSTER (same limits): a cluster of
 * six CTAs per ciphertext, one per (accumulator row, RNS channel), with one warp per digit
 * level, so no SM scheduler runs more than one transform: the shortest latency for lone
 * ciphertexts (six CTAs per ciphertext, no persistent grid). */
#define YG_LAYOUT_CHANNEL 0
#define YG_LAYOUT_CHANNEL_ROW 1
#define YG_LAYOUT_ROW_CLUSTER 2
#define YG_LAYOUT_CHANNEL_CLUSTER 3
/* Launch shape for this plan: layout, per_cta ciphertexts per blind-rotation CTA (1, 2 or
 * 4; 0 = the context's setting, layout included) and grid CTAs (0 = enough for the batch;
 * fewer = persistent CTAs that loop over it). */
int yg_plan_set_launch(yg_plan* plan, int layout, int per_cta, int grid);
int yg_plan_run(yg_plan* plan, const int32_t* d_in, int32_t* d_out, void* stream);
void yg_plan_destroy(yg_plan* plan);
/* Blind-rotation CTAs of per_cta ciphertexts each, in `layout`, that fit on one SM
 * (0: none fits, or no such kernel). */
int yg_ctas_per_sm(yg_ctx* ctx, int layout, int per_cta, int* out);
/* Launch shape of every bootstrap on this context (the autotuner's choice): layout,
 * per_cta ciphertexts per CTA (sharing its L1); ctas_per_sm > 0 makes the grid persistent
 * with that many CTAs per SM, 0 launches one CTA per group of per_cta ciphertexts.
 * Default (YG_LAYOUT_CHANNEL, 1, 0), except that until this is called a batch of at most
 * two waves of six-CTA clusters (48 ciphertexts on a 152-SM GPU) runs in
 * YG_LAYOUT_CHANNEL_CLUSTER where the parameters have it (one ciphertext alone: about a
 * sixth of the channel layout's time); after a call the shape given applies to every batch. */
int yg_ctx_set_launch(yg_ctx* ctx, int layout, int per_cta, int ctas_per_sm);

/* Serving: a request loop over many tenants with continuous batching and an HBM key cache.
 * Replaces the reference's CPU serving harness (ya_benchmark/blindrotate_serving.cpp:111-354,
 * ya_benchmark/include/blindrotate_serving.h:25-350) for the GINX method: the keys of
 * registered tenants are kept in pinned host memory in the device layout; at most
 * floor(key_budget_bytes / per-tenant key bytes) of them are resident in HBM at a time (an
 * LRU over tenants with no batch in flight), refilled on a miss by an asynchronous copy on
 * a side stream.  One worker thread admits pending requests, in arrival order, into
 * batches of up to max_batch ciphertexts while up to max_inflight earlier batches run (a
 * request larger than what is left of a batch is split across it and the next; it
 * completes with its last part); a batch bootstraps every request's ciphertexts with its
 * tenant's key and LUT.  Request buffers should be
 * pinned host memory (pageable buffers serialise the copies). */
typedef struct yg_server yg_server;
typedef struct yg_server_config {
    size_t key_budget_bytes;
    int max_batch;
    int max_inflight;
    int max_tenants;
    /* Batches of at most this many ciphertexts run in YG_LAYOUT_CHANNEL_CLUSTER where the
     * parameters have it (GINX keys, T = 32, N = 1024, l_approx <= 4): a lone ciphertext takes
     * about a third of the time of the throughput layouts.  0: two waves of the six-CTA
     * clusters the GPU holds at once; negative: never. */
    int latency_batch_max;
} yg_server_config;
typedef struct yg_server_counters {
    uint64_t key_hits, key_misses, refill_bytes, batches, requests_done, ciphertexts_done;
    int key_slots;
    uint64_t latency_batches; /* batches run in the latency layout (latency_batch_max) */
} yg_server_counters;
typedef struct yg_request_times {
    double t_submit, t_start, t_done; /* seconds on a monotonic clock */
} yg_request_times;
int yg_server_create(yg_ctx* ctx, const yg_server_config* cfg, yg_server** out);
/* Snapshots `key` (BSK + KSK, device layout) into pinned host memory; the key object may be
 * destroyed afterwards.  The first tenant fixes the server's key family: GINX rows (keys
 * made from GINX or WWL+24 words share one cache) or lazy keys, whose HBM slots hold only the
 * half rows and the s2 key (about a third of the GINX rows' bytes at the reference's default
 * 32-bit set, so the same key_budget_bytes holds that many more tenants) and whose batches
 * run the lazy blind rotation; a tenant of the other family is refused with YG_ERR_INVALID,
 * as are group keys.  A budget smaller than one tenant's keys is refused here.  h_lut: the
 * tenant's test polynomial ([N] int64). */
int yg_server_add_tenant(yg_server* s, int tenant, const yg_key* key, const int64_t* h_lut);
int yg_server_start(yg_server* s);
/* Returns a request id (> 0) or a negative status. */
int64_t yg_server_submit(yg_server* s, int tenant, const int32_t* h_in, int32_t* h_out, int count);
int yg_server_wait(yg_server* s, int64_t request, int timeout_ms, yg_request_times* times);
int yg_server_stats(yg_server* s, yg_server_counters* out);
void yg_server_destroy(yg_server* s);

/* A whole serving trace, generated and timed inside the library: `requests` arrivals of a
 * Poisson process at `rate` requests/s (exponential gaps from mt19937_64(seed ^
 * 0x9e3779b97f4a7c15), as blindrotate_serving.cpp:184), tenants 0..tenants-1 drawn from
 * Zipf(zipf_s) (ZipfDistribution, yatfhe/include/yautil/zipf.h:47-87, seeded zipf_seed),
 * sizes floor(exp(U(0, ln(max_count + 1)))) clamped to [1, max_count].  Request r of tenant t
 * bootstraps rows [0, size) of h_pool[t] ([tenants][max_count][n+1] pinned); when h_expect
 * (same shape) is given every output is compared with it.  The first `warmup` requests are
 * served but not measured.  Latencies (ms) are ceil-rank percentiles. */
typedef struct yg_trace_config {
    int requests, warmup;
    double rate;
    uint64_t seed;
    double zipf_s;
    uint64_t zipf_seed;
    int tenants;
    int max_count;
    int queue_max; /* arrivals that find more requests than this unfinished are shed (0 = no bound) */
    const int32_t* h_pool;
    const int32_t* h_expect;
    double slo_ms; /* sojourn target of slo_violation_rate (0 = 100 ms, the reference's default) */
} yg_trace_config;
typedef struct yg_latency {
    double mean_ms, p50_ms, p90_ms, p99_ms, p999_ms, max_ms;
} yg_latency;
typedef struct yg_trace_result {
    int served, shed, mismatched_requests;
    double seconds, requests_per_s, ciphertexts_per_s, offered_rate;
    yg_latency sojourn, queue, service;
    uint64_t key_hits, key_misses, refill_bytes, batches;
    double hit_rate;
    /* The reference harness's figures (ya_benchmark/blindrotate_serving.cpp:256-284, 324-336),
     * over the measured requests: the share whose sojourn exceeds slo_ms and 100 / 300 / 500 ms;
     * Jain's index of the tenants' mean sojourn times, (sum m)^2 / (tenants * sum m^2), 1 =
     * every tenant waits the same; the most requests submitted and not yet started at once;
     * key refills belonging to batches not yet finished, the most at once and the mean over
     * batch launches. */
    double slo_ms, slo_violation_rate, slo_violation_rate_100, slo_violation_rate_300, slo_violation_rate_500;
    double tenant_fairness_jain;
    int peak_queue_depth, load_concurrency_peak;
    double load_concurrency_mean;
    uint64_t latency_batches; /* of `batches`, those run in the latency layout */
} yg_trace_result;
int yg_server_run_trace(yg_server* s, const yg_trace_config* cfg, yg_trace_result* out);

/* Health counter, no reference counterpart: how many bounded waits inside this library's
 * kernels on ctx's device gave up since the library was loaded (the row-cluster layout's
 * wait for its TMA key copies; the kernel then reads the key from global memory, so results
 * stay correct).  0 in normal operation. */
int yg_wait_timeouts(yg_ctx* ctx, uint64_t* out);

/* Calibration, no reference counterpart: measured 32-bit multiply-add throughput of
 * `device` (operations per second), the denominator of the bootstrap's roofline. */
int yg_probe_int32_rate(int device, double* ops_per_second);

#ifdef __cplusplus
}
#endif

#endif /* YATFHE_GB300_H */
