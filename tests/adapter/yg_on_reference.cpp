// yg_on_reference.cpp -- TEST INFRASTRUCTURE ONLY.  A CPU stand-in for the part of the GB300
// C ABI (include/yatfhe_gb300.h) that the C++ adapter (include/yatfhe_gb300_reference.hpp)
// calls for GINX keys, built on the reference's own functions, plus host-memory versions of
// the three CUDA memory calls the adapter makes.  Each entry point rebuilds the reference's
// objects from the flat buffers the adapter produced and calls the reference function the
// real entry point replaces; so a program that runs the adapter against this file gets the
// reference's own result exactly when the adapter's conversions (word order, levels, rows,
// signs, widths, the key cache) are right.  The CUDA side of the same ABI is checked by the
// GPU tests.  Linked only into tests/adapter/adapter_run.cpp.
#include <cuda_runtime_api.h>

#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "yatfhe/blind_rotate.h"
#include "yatfhe/bootstrapping.h"
#include "yatfhe/keyswitching.h"
#include "yatfhe/ntt24.h"
#include "yatfhe/trgsw.h"
#include "yatfhe/tlwe.h"
#include "yatfhe/trlwe.h"
#include "yatfhe_gb300.h"

struct yg_ctx {
    yg_params p;
};

struct yg_key {
    std::unique_ptr<BootstrappingKeyMP> bsk;
    std::unique_ptr<TlweKeySwitchingKey> ksk;
    std::unique_ptr<BootstrappingKeyMPLazyPipeAlt> lazy;
};

struct yg_crt_key {
    std::unique_ptr<BootstrappingKeyCRT> bsk;
};

namespace {

const YatfheParameters* g_param = nullptr;
thread_local std::string g_err;
int g_uploads = 0;  // GINX key uploads (adapter_run.cpp checks the adapter's key cache with it)
int g_crt_uploads = 0;

int fail(int rc, const std::string& what) {
    g_err = what;
    return rc;
}

}  // namespace

extern "C" {

// the process-wide parameters the reference functions run with (adapter_run.cpp's initYatfhe)
void yg_test_use_params(const YatfheParameters* p) { g_param = p; }
int yg_test_uploads(void) { return g_uploads; }
int yg_test_crt_uploads(void) { return g_crt_uploads; }

const char* yg_last_error(void) { return g_err.c_str(); }

int yg_ctx_create(const yg_params* q, int device, yg_ctx** out) {
    const YatfheParameters& p = *g_param;
    if (device != 0) return fail(YG_ERR_INVALID, "device");
    if (q->n != p.n || q->N != p.N || q->k != p.k || q->radix_bits != p.radixBits || q->l_approx != p.lApprox ||
        q->ks_radix_bits != p.ksRadixBits || q->ks_level != p.ksLevel || q->torus_bits != p.torusBits)
        return fail(YG_ERR_INVALID, "parameters differ from the reference's");
    *out = new yg_ctx{*q};
    return YG_OK;
}

void yg_ctx_destroy(yg_ctx* c) { delete c; }

// [n][l][k+1][k+1][N] words -> BootstrappingKeyMP::bskDft
int yg_key_upload_bsk_ntt(yg_ctx* c, const uint64_t* w, yg_key** out) {
    const YatfheParameters& p = *g_param;
    auto key = std::make_unique<yg_key>();
    key->bsk = std::make_unique<BootstrappingKeyMP>(p, c->p.l_approx);
    size_t o = 0;
    for (auto& g : key->bsk->bskDft) {
        TrgswMPDft& t = g[0];
        for (int lvl = 0; lvl < t.l; lvl++)
            for (int row = 0; row <= p.k; row++) {
                TrlweDft& r = row < p.k ? t.c[lvl][row] : t.cPrime[lvl];
                for (int poly = 0; poly <= p.k; poly++) {
                    NttPolynomial& P = poly < p.k ? r.a[poly] : r.b;
                    std::memcpy(P.coeffs.data(), w + o, sizeof(uint64_t) * p.N);
                    o += p.N;
                }
            }
    }
    g_uploads++;
    *out = key.release();
    return YG_OK;
}

int yg_key_create_ksk_only(yg_ctx*, yg_key** out) {
    *out = new yg_key{};
    return YG_OK;
}

// [k N][t][n + 1] int32 words -> TlweKeySwitchingKey::decomposedKsk
int yg_key_set_ksk(yg_key* key, const int32_t* w) {
    const YatfheParameters& p = *g_param;
    key->ksk = std::make_unique<TlweKeySwitchingKey>(p);
    size_t o = 0;
    for (auto& row : key->ksk->decomposedKsk)
        for (auto& t : row) {
            for (int i = 0; i < p.n; i++) t.a[i] = static_cast<LweTorus>(w[o + i]);
            t.b = static_cast<LweTorus>(w[o + p.n]);
            o += p.n + 1;
        }
    return YG_OK;
}

void yg_key_destroy(yg_key* key) { delete key; }

// functionalBootstrappingMPNtt per ciphertext (yatfhe/src/bootstrapping.cpp:71-80)
int yg_pbs_host(yg_ctx*, const yg_key* key, const int32_t* in, int32_t* out, int count, const int64_t* lut, void*) {
    const YatfheParameters& p = *g_param;
    if (!key->bsk || !key->ksk) return fail(YG_ERR_STATE, "no key");
    TorusPolynomial v{p.N};
    for (int j = 0; j < p.N; j++) v.coeffs[j] = static_cast<Torus>(lut[j]);
    for (int c = 0; c < count; c++) {
        Tlwe x{p.n}, y{p.n};
        const int32_t* w = in + static_cast<size_t>(c) * (p.n + 1);
        for (int i = 0; i < p.n; i++) x.a[i] = static_cast<LweTorus>(w[i]);
        x.b = static_cast<LweTorus>(w[p.n]);
        functionalBootstrappingMPNtt(y, x, *key->bsk, *key->ksk, v, p);
        int32_t* o = out + static_cast<size_t>(c) * (p.n + 1);
        for (int i = 0; i < p.n; i++) o[i] = static_cast<int32_t>(y.a[i]);
        o[p.n] = static_cast<int32_t>(y.b);
    }
    return YG_OK;
}

// blindRotateMP21Ntt in place (yatfhe/src/blind_rotate.cpp:1538-1565)
int yg_blind_rotate_acc(yg_ctx*, const yg_key* key, const int32_t* scaled, int64_t* acc, int count, void*) {
    const YatfheParameters& p = *g_param;
    for (int c = 0; c < count; c++) {
        ScaledTlwe s{2 * p.N, p.n};
        for (int i = 0; i < p.n; i++) s.a[i] = scaled[static_cast<size_t>(c) * p.n + i];
        Trlwe t{p.k, p.N};
        int64_t* a = acc + static_cast<size_t>(c) * (p.k + 1) * p.N;
        for (int r = 0; r < p.k; r++)
            for (int j = 0; j < p.N; j++) t.a[r].coeffs[j] = static_cast<Torus>(a[static_cast<size_t>(r) * p.N + j]);
        for (int j = 0; j < p.N; j++) t.b.coeffs[j] = static_cast<Torus>(a[static_cast<size_t>(p.k) * p.N + j]);
        blindRotateMP21Ntt(t, key->bsk->bskDft, s, p);
        for (int r = 0; r < p.k; r++)
            for (int j = 0; j < p.N; j++) a[static_cast<size_t>(r) * p.N + j] = static_cast<int64_t>(t.a[r].coeffs[j]);
        for (int j = 0; j < p.N; j++) a[static_cast<size_t>(p.k) * p.N + j] = static_cast<int64_t>(t.b.coeffs[j]);
    }
    return YG_OK;
}

// switchKeyForTlwe (yatfhe/src/keyswitching.cpp:48-72)
int yg_keyswitch(yg_ctx*, const yg_key* key, const int32_t* big, int32_t* out, int count, void*) {
    const YatfheParameters& p = *g_param;
    const int kN = p.k * p.N;
    for (int c = 0; c < count; c++) {
        Tlwe x{kN}, y{p.n};
        const int32_t* w = big + static_cast<size_t>(c) * (kN + 1);
        for (int i = 0; i < kN; i++) x.a[i] = static_cast<LweTorus>(w[i]);
        x.b = static_cast<LweTorus>(w[kN]);
        switchKeyForTlwe(y, *key->ksk, x, p);
        int32_t* o = out + static_cast<size_t>(c) * (p.n + 1);
        for (int i = 0; i < p.n; i++) o[i] = static_cast<int32_t>(y.a[i]);
        o[p.n] = static_cast<int32_t>(y.b);
    }
    return YG_OK;
}

// half rows [n][L][k+1][N] (torus values) + s2 key [Ls][k+1][N] (NTT words) ->
// BootstrappingKeyMPLazyPipeAlt
int yg_key_upload_lazy(yg_ctx* c, const int64_t* cprime, const uint64_t* s2, int s2_levels, yg_key** out) {
    const YatfheParameters& p = *g_param;
    if (s2_levels != p.l) return fail(YG_ERR_INVALID, "s2 levels");
    auto key = std::make_unique<yg_key>();
    key->lazy = std::make_unique<BootstrappingKeyMPLazyPipeAlt>(p, c->p.l_approx, true);
    size_t o = 0;
    for (auto& t : key->lazy->bskPrime)
        for (int lvl = 0; lvl < c->p.l_approx; lvl++)
            for (int poly = 0; poly <= p.k; poly++) {
                TorusPolynomial& P = poly < p.k ? t.cPrime[lvl].a[poly] : t.cPrime[lvl].b;
                for (int j = 0; j < p.N; j++) P.coeffs[j] = static_cast<Torus>(cprime[o++]);
            }
    o = 0;
    for (auto& t : key->lazy->s2Dft.trlweDfts)
        for (int poly = 0; poly <= p.k; poly++) {
            NttPolynomial& P = poly < p.k ? t.a[poly] : t.b;
            std::memcpy(P.coeffs.data(), s2 + o, sizeof(uint64_t) * p.N);
            o += p.N;
        }
    g_uploads++;
    *out = key.release();
    return YG_OK;
}

// the whole blind rotation from the test polynomial (lazy keys: blindRotateLazyPipeAltNtt,
// which builds its accumulator from v and the input itself)
int yg_blind_rotate(yg_ctx*, const yg_key* key, const int32_t* in, const int64_t* lut, int64_t* acc, int count,
                    int steps, void*) {
    const YatfheParameters& p = *g_param;
    if (!key->lazy || steps != p.n) return fail(YG_ERR_INVALID, "stand-in: lazy keys, whole rotations only");
    const int n = p.n, N = p.N, k = p.k;
    TorusPolynomial v{N};
    for (int j = 0; j < N; j++) v.coeffs[j] = static_cast<Torus>(lut[j]);
    std::vector<NttPolynomial> gdV;
    prepareGdV(gdV, v, p);
    for (int c = 0; c < count; c++) {
        Tlwe x{n};
        const int32_t* w = in + static_cast<size_t>(c) * (n + 1);
        for (int i = 0; i < n; i++) x.a[i] = static_cast<LweTorus>(w[i]);
        x.b = static_cast<LweTorus>(w[n]);
        ScaledTlwe sc{2 * N, n};
        rescaleTlweToNewMod(sc, x);
        Trlwe a{k, N};
        blindRotateLazyPipeAltNtt(a, *key->lazy, sc, v, gdV, p);
        int64_t* o = acc + static_cast<size_t>(c) * (k + 1) * N;
        for (int r = 0; r < k; r++)
            for (int j = 0; j < N; j++) o[static_cast<size_t>(r) * N + j] = static_cast<int64_t>(a.a[r].coeffs[j]);
        for (int j = 0; j < N; j++) o[static_cast<size_t>(k) * N + j] = static_cast<int64_t>(a.b.coeffs[j]);
    }
    return YG_OK;
}

// residue rows [n][d][dh][k+1][k+1][N] -> BootstrappingKeyCRT (bsk8 and its NTT24 forms)
int yg_crt_key_upload(int device, int n, int N, const int8_t* h, yg_crt_key** out) {
    const YatfheParameters& p = *g_param;
    if (device != 0 || n != p.n || N != p.N) return fail(YG_ERR_INVALID, "ApproxCRT key shape");
    auto key = std::make_unique<yg_crt_key>();
    key->bsk = std::make_unique<BootstrappingKeyCRT>(p);
    size_t o = 0;
    for (int i = 0; i < p.n; i++)
        for (int d = 0; d < p.d; d++) {
            for (int l = 0; l < p.dh; l++)
                for (int r = 0; r <= p.k; r++) {
                    Trlwe8& t = key->bsk->bsk8[i][d].trlweSamples[l][r];
                    for (int c = 0; c <= p.k; c++) {
                        Int8Polynomial& P = c < p.k ? t.a[c] : t.b;
                        std::memcpy(P.coeffs.data(), h + o, p.N);
                        o += p.N;
                    }
                }
            NttNative24::applyNttForRgsw(key->bsk->bskCRT[i][d], key->bsk->bsk8[i][d]);
        }
    g_crt_uploads++;
    *out = key.release();
    return YG_OK;
}

// decompTrlweMcrt, blindRotateApproxCRTNtt, trlweMcrtToCrt, recompTrlweCrt per ciphertext
int yg_crt_blind_rotate(yg_crt_key* key, const int32_t* in, const int32_t* rot, int count, int32_t* out, void*) {
    const YatfheParameters& p = *g_param;
    const int N = p.N;
    for (int c = 0; c < count; c++) {
        Trlwe t{p.k, N};
        const int32_t* w = in + static_cast<size_t>(c) * 2 * N;
        for (int j = 0; j < N; j++) {
            t.a[0].coeffs[j] = static_cast<Torus>(w[j]);
            t.b.coeffs[j] = static_cast<Torus>(w[N + j]);
        }
        ScaledTlwe s{2 * N, p.n};
        for (int i = 0; i < p.n; i++) s.a[i] = rot[static_cast<size_t>(c) * p.n + i];
        std::vector<Trlwe8> acc(p.d, Trlwe8{p.k, N});
        decompTrlweMcrt(acc, t, p);
        blindRotateApproxCRTNtt(acc, key->bsk->bskCRT, s, p);
        trlweMcrtToCrt(acc, p);
        Trlwe r{p.k, N};
        recompTrlweCrt(r, acc, p);
        int32_t* o = out + static_cast<size_t>(c) * 2 * N;
        for (int j = 0; j < N; j++) {
            o[j] = static_cast<int32_t>(r.a[0].coeffs[j]);
            o[N + j] = static_cast<int32_t>(r.b.coeffs[j]);
        }
    }
    return YG_OK;
}

void yg_crt_key_destroy(yg_crt_key* key) { delete key; }

// "device" memory of this stand-in: host memory
cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::malloc(n ? n : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, enum cudaMemcpyKind) {
    std::memcpy(dst, src, n);
    return cudaSuccess;
}
const char* cudaGetErrorString(cudaError_t) { return "stand-in CUDA error"; }

}  // extern "C"
