// ref_capi.cpp -- a flat C API over the reference library's own functions, compiled
// together with the reference's sources into oracle/_ref/libyatfhe_ref_t{32,56}.so.
// TEST INFRASTRUCTURE ONLY: the tests use it to pin the plain-C restatement
// (oracle/pbs_oracle.c) and the GPU path against the reference itself, and the CPU
// baseline times functionalBootstrappingMPNtt through it.  Every entry point below just
// marshals flat buffers into the reference's types and calls the reference function
// named in its comment; no arithmetic of the bootstrap path lives here.
//
// Buffers: torus values cross this API as int64 (sign-extended), LWE ciphertexts as
// int32 words [a_0 .. a_{n-1}, b] (the reference keeps them mod 2^32, in int64 under
// TORUS56, yatfhe/include/yatfhe/torus.h:24-30).
#include <cstdint>
#include <cstring>
#include <exception>
#include <future>
#include <string>
#include <vector>

#include "yatfhe/blind_rotate.h"
#include "yatfhe/bootstrapping.h"
#include "yatfhe/crt.h"
#include "yatfhe/ntt24.h"
#include "yatfhe/gadget_decomposition.h"
#include "yatfhe/keyswitching.h"
#include "yatfhe/ntt_hexl.h"
#include "yatfhe/numeric.h"
#include "yatfhe/polynomial.h"
#include "yatfhe/tlwe.h"
#include "yatfhe/trgsw.h"
#include "yatfhe/trlev.h"
#include "yatfhe/trlwe.h"
#include "yautil/initializer.h"
#include "yautil/multi_threading.h"
#include "yautil/ya_serializer.h"

extern "C" void yatfhe_oracle_set_seed(uint64_t seed);

namespace {

struct RefState {
    YatfheParameters param{};
    bool ready{false};
    std::unique_ptr<TlweKey> lweKey;
    std::unique_ptr<TrgswKey> trgswKey;
    std::unique_ptr<BootstrappingKeyMP> bsk;
    std::unique_ptr<BootstrappingKeyWWL24> wwl;
    std::unique_ptr<BootstrappingKeyMPLazyPipeAlt> lazy;
    std::unique_ptr<BootstrappingKey> gbsk;  // the group-g key family (TrgswDft rows)
    std::unique_ptr<TlweKeySwitchingKey> ksk;
    std::string lastError;
};

RefState& st() {
    static RefState s;
    return s;
}

int fail(const char* what) {
    st().lastError = what;
    return -1;
}

template <typename F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        st().lastError = e.what();
        return -1;
    }
}

void toTlwe(Tlwe& t, const int32_t* w, int n) {
    for (int i = 0; i < n; i++) t.a[i] = static_cast<LweTorus>(w[i]);
    t.b = static_cast<LweTorus>(w[n]);
}

void fromTlwe(int32_t* w, const Tlwe& t, int n) {
    for (int i = 0; i < n; i++) w[i] = static_cast<int32_t>(t.a[i]);
    w[n] = static_cast<int32_t>(t.b);
}

void toPoly(TorusPolynomial& p, const int64_t* v, int N) {
    for (int j = 0; j < N; j++) p.coeffs[j] = static_cast<Torus>(v[j]);
}

void fromPoly(int64_t* v, const TorusPolynomial& p, int N) {
    for (int j = 0; j < N; j++) v[j] = static_cast<int64_t>(p.coeffs[j]);
}

}  // namespace

extern "C" {

struct ref_params {
    int n, N, k, radix_bits, l, l_approx, ks_radix_bits, ks_level, lwe_noise_b, rlwe_noise_b, torus_base;
};

const char* ref_last_error(void) { return st().lastError.c_str(); }

int ref_torus_bits(void) { return static_cast<int>(sizeof(Torus) == 4 ? 32 : 56); }

// YatfheParameters (yatfhe/include/yatfhe/yatfhe_parameters.h:9-110) + initYatfhe
// (yatfhe/src/initializer.cpp:50-85).
int ref_setup(const ref_params* p) {
    return guarded([&] {
        auto& s = st();
        s.param = YatfheParameters{};
        auto& q = s.param;
        q.n = p->n;
        q.N = p->N;
        q.k = p->k;
        q.setRadixBits(p->radix_bits);
        q.l = p->l;
        q.lApprox = p->l_approx;
        q.setKsRadixBits(p->ks_radix_bits);
        q.ksLevel = p->ks_level;
        q.lweNoiseB = p->lwe_noise_b;
        q.rlweNoiseB = p->rlwe_noise_b;
        q.torusBase = p->torus_base;
        initYatfhe(q);
        s.lweKey.reset();
        s.trgswKey.reset();
        s.bsk.reset();
        s.wwl.reset();
        s.lazy.reset();
        s.gbsk.reset();
        s.ksk.reset();
        s.ready = true;
    });
}

// Key generation, all on the calling thread's RNG stream 0: genTlweKey
// (yatfhe/src/tlwe.cpp:10-18), genTrlweKey (yatfhe/src/trlwe.cpp:70-81), then the per-i
// body of genBootstrappingKeyMP (yatfhe/src/bootstrapping.cpp:150-174), i.e.
// encryptTrgswMPNtt(bskDft[i][0], s_i, ...) for i = 0..n-1 in order, then
// genTlweKeySwitchingKey (yatfhe/src/keyswitching.cpp:19-29).  The reference runs the
// BSK loop on its thread pool, which makes the RNG stream per worker; running the same
// per-i calls in order keeps one stream and so one key per seed.
int ref_keygen(uint64_t seed) {
    if (!st().ready) return fail("ref_keygen: ref_setup not called");
    return guarded([&] {
        auto& s = st();
        auto& p = s.param;
        (void)rng();  // construct this thread's instance before reseeding it
        yatfhe_oracle_set_seed(seed);
        rng = ChaCha20Rng();
        s.lweKey = std::make_unique<TlweKey>(p);
        s.trgswKey = std::make_unique<TrgswKey>(p);
        s.bsk = std::make_unique<BootstrappingKeyMP>(p, p.lApprox);
        s.ksk = std::make_unique<TlweKeySwitchingKey>(p);
        genTlweKey(*s.lweKey);
        genTrlweKey(s.trgswKey->trlweKey);
        for (int i = 0; i < s.bsk->n; i++) {
            encryptTrgswMPNtt(s.bsk->bskDft[i][0], s.lweKey->s[i], *s.trgswKey, 0, p);
        }
        TlweKey ksTarget = *s.lweKey;
        genTlweKeySwitchingKey(*s.ksk, s.trgswKey->trlweKey, ksTarget, p);
    });
}

// serializeBskMP / deserializeBskMP (yatfhe/src/ya_serializer.cpp:276-303).
int ref_save_bsk(const char* path) {
    if (!st().bsk) return fail("ref_save_bsk: no key");
    return guarded([&] { serializeBskMP(*st().bsk, path); });
}

int ref_load_bsk(const char* path) {
    if (!st().ready) return fail("ref_load_bsk: ref_setup not called");
    return guarded([&] {
        auto& s = st();
        s.bsk = std::make_unique<BootstrappingKeyMP>();
        deserializeBskMP(*s.bsk, path, s.param.n);
    });
}

// NTT-domain words of the loaded BSK as [i][lvl][row][poly][N], row = c[lvl][0..k-1]
// then cPrime[lvl], poly = a[0..k-1] then b (TrgswMPDft, yatfhe/include/yatfhe/trgsw.h:45-87).
int ref_export_bsk_ntt(uint64_t* out) {
    if (!st().bsk) return fail("ref_export_bsk_ntt: no key");
    auto& s = st();
    const int k = s.param.k, N = s.param.N;
    size_t o = 0;
    for (int i = 0; i < s.bsk->n; i++) {
        const auto& g = s.bsk->bskDft[i][0];
        for (int lvl = 0; lvl < g.l; lvl++) {
            for (int row = 0; row <= k; row++) {
                const TrlweDft& r = row < k ? g.c[lvl][row] : g.cPrime[lvl];
                for (int poly = 0; poly <= k; poly++) {
                    const NttPolynomial& P = poly < k ? r.a[poly] : r.b;
                    std::memcpy(out + o, P.coeffs.data(), sizeof(uint64_t) * N);
                    o += N;
                }
            }
        }
    }
    return 0;
}

int ref_export_keys(int32_t* lwe_s, int32_t* rlwe_s) {
    auto& s = st();
    if (!s.lweKey || !s.trgswKey) return fail("ref_export_keys: no key");
    for (int i = 0; i < s.param.n; i++) lwe_s[i] = static_cast<int32_t>(s.lweKey->s[i]);
    for (int r = 0; r < s.param.k; r++)
        for (int j = 0; j < s.param.N; j++)
            rlwe_s[r * s.param.N + j] = static_cast<int32_t>(s.trgswKey->trlweKey.s[r].coeffs[j]);
    return 0;
}

int ref_import_keys(const int32_t* lwe_s, const int32_t* rlwe_s) {
    auto& s = st();
    if (!s.ready) return fail("ref_import_keys: ref_setup not called");
    return guarded([&] {
        s.lweKey = std::make_unique<TlweKey>(s.param);
        s.trgswKey = std::make_unique<TrgswKey>(s.param);
        for (int i = 0; i < s.param.n; i++) s.lweKey->s[i] = lwe_s[i];
        for (int r = 0; r < s.param.k; r++) {
            for (int j = 0; j < s.param.N; j++) s.trgswKey->trlweKey.s[r].coeffs[j] = rlwe_s[r * s.param.N + j];
            NttHexl::applyNtt(s.trgswKey->trlweKey.sDft[r], s.trgswKey->trlweKey.s[r]);
        }
    });
}

// TlweKeySwitchingKey decomposedKsk[kN][t] of Tlwe(n) (yatfhe/include/yatfhe/keyswitching.h:14-31)
// as int32 words [i][j][n+1].
int ref_export_ksk(int32_t* out) {
    auto& s = st();
    if (!s.ksk) return fail("ref_export_ksk: no key");
    const int n = s.param.n;
    size_t o = 0;
    for (const auto& row : s.ksk->decomposedKsk)
        for (const auto& t : row) {
            fromTlwe(out + o, t, n);
            o += n + 1;
        }
    return 0;
}

int ref_import_ksk(const int32_t* in) {
    auto& s = st();
    if (!s.ready) return fail("ref_import_ksk: ref_setup not called");
    return guarded([&] {
        s.ksk = std::make_unique<TlweKeySwitchingKey>(s.param);
        const int n = s.param.n;
        size_t o = 0;
        for (auto& row : s.ksk->decomposedKsk)
            for (auto& t : row) {
                toTlwe(t, in + o, n);
                o += n + 1;
            }
    });
}

// symEncTlwe (yatfhe/src/tlwe.cpp:21-31) on this thread's RNG stream, one call per message.
int ref_encrypt(const int64_t* mu, int count, int32_t* out) {
    auto& s = st();
    if (!s.lweKey) return fail("ref_encrypt: no key");
    const int n = s.param.n;
    Tlwe t{n};
    for (int c = 0; c < count; c++) {
        symEncTlwe(t, static_cast<Torus>(mu[c]), *s.lweKey);
        fromTlwe(out + static_cast<size_t>(c) * (n + 1), t, n);
    }
    return 0;
}

// symDecTlweToInt (yatfhe/src/tlwe.cpp:44-53).
int ref_decrypt(const int32_t* in, int count, int base, int32_t* out) {
    auto& s = st();
    if (!s.lweKey) return fail("ref_decrypt: no key");
    const int n = s.param.n;
    Tlwe t{n};
    for (int c = 0; c < count; c++) {
        toTlwe(t, in + static_cast<size_t>(c) * (n + 1), n);
        out[c] = static_cast<int32_t>(symDecTlweToInt(t, *s.lweKey, base));
    }
    return 0;
}

// generateTestPolynomial (kind 0) / generateTestPolynomialFR (kind 1)
// (yatfhe/src/polynomial.cpp:75-107), with modQ = 2N.
int ref_test_polynomial(int kind, int modP, int64_t* v) {
    auto& s = st();
    const int N = s.param.N;
    TorusPolynomial p{N};
    if (kind == 0) generateTestPolynomial(p, modP, 2 * N);
    else generateTestPolynomialFR(p, modP, 2 * N);
    fromPoly(v, p, N);
    return 0;
}

// rescaleTlweToNewMod (yatfhe/src/tlwe.cpp:75-81) into mod 2N; out = [a_0..a_{n-1}, b].
int ref_modswitch(const int32_t* in, int32_t* out) {
    auto& s = st();
    const int n = s.param.n;
    Tlwe t{n};
    toTlwe(t, in, n);
    ScaledTlwe sc{2 * s.param.N, n};
    rescaleTlweToNewMod(sc, t);
    for (int i = 0; i < n; i++) out[i] = sc.a[i];
    out[n] = sc.b;
    return 0;
}

// rotateTorusPolynomial / rotateTorusPolynomialMinusOne (yatfhe/src/polynomial.cpp:184-238).
int ref_rotate(const int64_t* in, int N, int a, int minus_one, int64_t* out) {
    TorusPolynomial x{N}, y{N};
    toPoly(x, in, N);
    if (minus_one) rotateTorusPolynomialMinusOne(y, a, x);
    else rotateTorusPolynomial(y, a, x);
    fromPoly(out, y, N);
    return 0;
}

// decomposeRow (yatfhe/include/yatfhe/gadget_decomposition.h:190-236) with `levels`
// levels; out = [level][N].
int ref_decompose(const int64_t* in, int N, int levels, int64_t* out) {
    return guarded([&] {
        std::vector<Torus> x(N);
        for (int j = 0; j < N; j++) x[j] = static_cast<Torus>(in[j]);
        std::vector<std::vector<Torus>> d(levels, std::vector<Torus>(N));
        std::vector<Torus*> ptr(levels);
        for (int l = 0; l < levels; l++) ptr[l] = d[l].data();
        decomposeRow(ptr.data(), x.data(), N, levels, st().param);
        for (int l = 0; l < levels; l++)
            for (int j = 0; j < N; j++) out[static_cast<size_t>(l) * N + j] = d[l][j];
    });
}

// signedGadgetDecompositionKs (yatfhe/src/gadget_decomposition.cpp:53-56); out = t digits.
int ref_decompose_ks(int64_t value, int64_t* out) {
    auto& p = st().param;
    DecomposedData d{p.ksLevel};
    signedGadgetDecompositionKs(d, static_cast<Torus>(value), p);
    for (int j = 0; j < p.ksLevel; j++) out[j] = static_cast<int64_t>(d.value[j]) * d.sign;
    return 0;
}

// NttHexl::applyNtt / applyIntt (yatfhe/include/yatfhe/ntt_hexl.h:34-44,
// yatfhe/src/ntt_hexl.cpp:153-175).
int ref_ntt_forward(const int64_t* in, uint64_t* out) {
    const int N = st().param.N;
    TorusPolynomial x{N};
    toPoly(x, in, N);
    NttPolynomial y{N};
    NttHexl::applyNtt(y, x);
    std::memcpy(out, y.coeffs.data(), sizeof(uint64_t) * N);
    return 0;
}

int ref_ntt_inverse(const uint64_t* in, int64_t* out) {
    const int N = st().param.N;
    NttPolynomial x{N};
    std::memcpy(x.coeffs.data(), in, sizeof(uint64_t) * N);
    TorusPolynomial y{N};
    NttHexl::applyIntt(y, x);
    fromPoly(out, y, N);
    return 0;
}

uint64_t ref_ntt_root(void) { return NttHexl::getNttHexl().GetMinimalRootOfUnity(); }

// externalProductTrgswMPNtt (yatfhe/src/trgsw.cpp:769-772) with BSK row i; trlwe = [a..., b].
int ref_external_product(const int64_t* in, int i, int64_t* out) {
    auto& s = st();
    if (!s.bsk) return fail("ref_external_product: no key");
    const int k = s.param.k, N = s.param.N;
    Trlwe x{k, N}, y{k, N};
    for (int r = 0; r < k; r++) toPoly(x.a[r], in + static_cast<size_t>(r) * N, N);
    toPoly(x.b, in + static_cast<size_t>(k) * N, N);
    const auto& g = s.bsk->bskDft[i][0];
    externalProductTrgswMPNtt(y, g, x, g.l, s.param);
    for (int r = 0; r < k; r++) fromPoly(out + static_cast<size_t>(r) * N, y.a[r], N);
    fromPoly(out + static_cast<size_t>(k) * N, y.b, N);
    return 0;
}

// extractTlweFromTrlwe(out, acc, 0) (yatfhe/src/trlwe.cpp:240-250); out has k*N + 1 words.
int ref_extract(const int64_t* acc, int32_t* out) {
    auto& s = st();
    const int k = s.param.k, N = s.param.N;
    Trlwe x{k, N};
    for (int r = 0; r < k; r++) toPoly(x.a[r], acc + static_cast<size_t>(r) * N, N);
    toPoly(x.b, acc + static_cast<size_t>(k) * N, N);
    Tlwe t{k * N};
    extractTlweFromTrlwe(t, x, s.param.driftPhase);
    fromTlwe(out, t, k * N);
    return 0;
}

// switchKeyForTlwe (yatfhe/src/keyswitching.cpp:48-72); in has k*N + 1 words, out n + 1.
int ref_keyswitch(const int32_t* in, int32_t* out) {
    auto& s = st();
    if (!s.ksk) return fail("ref_keyswitch: no key");
    const int n = s.param.n, kN = s.param.k * s.param.N;
    Tlwe x{kN}, y{n};
    toTlwe(x, in, kN);
    switchKeyForTlwe(y, *s.ksk, x, s.param);
    fromTlwe(out, y, n);
    return 0;
}

// rescaleTlweToNewMod + genNoiselessTrlweSample + the MP21 loop body
// (yatfhe/src/blind_rotate.cpp:1556-1563) replayed through the public functions
// rotateTrlweMinusOne / externalProductTrgswMPNttInPlace / accumulateTrlwe, writing the
// accumulator [a..., b] after every iteration listed in `checkpoints` (ascending, each in
// [0, n)).  The final accumulator is also recomputed by blindRotateMP21Ntt itself and
// the call fails if the two disagree.
int ref_blind_rotate_trace(const int32_t* in, const int64_t* v, const int* checkpoints, int ncheck, int64_t* acc_out,
                           int64_t* acc_final) {
    auto& s = st();
    if (!s.bsk) return fail("ref_blind_rotate_trace: no key");
    const auto& p = s.param;
    const int n = p.n, k = p.k, N = p.N;
    Tlwe t{n};
    toTlwe(t, in, n);
    ScaledTlwe sc{2 * N, n};
    rescaleTlweToNewMod(sc, t);
    TorusPolynomial vp{N};
    toPoly(vp, v, N);
    Trlwe acc{k, N}, tmp{k, N}, acc2{k, N};
    genNoiselessTrlweSample(acc, vp, sc);
    genNoiselessTrlweSample(acc2, vp, sc);
    const int level = s.bsk->bskDft[0][0].l;
    int c = 0;
    const size_t stride = static_cast<size_t>(k + 1) * N;
    for (int i = 0; i < n; i++) {
        if (sc.a[i] != 0) {
            rotateTrlweMinusOne(tmp, acc, sc.a[i]);
            externalProductTrgswMPNttInPlace(tmp, s.bsk->bskDft[i][0], level, p);
            accumulateTrlwe(acc, tmp);
        }
        while (c < ncheck && checkpoints[c] == i) {
            for (int r = 0; r < k; r++) fromPoly(acc_out + c * stride + static_cast<size_t>(r) * N, acc.a[r], N);
            fromPoly(acc_out + c * stride + static_cast<size_t>(k) * N, acc.b, N);
            c++;
        }
    }
    blindRotateMP21Ntt(acc2, s.bsk->bskDft, sc, p);
    for (int r = 0; r < k; r++) fromPoly(acc_final + static_cast<size_t>(r) * N, acc2.a[r], N);
    fromPoly(acc_final + static_cast<size_t>(k) * N, acc2.b, N);
    for (int r = 0; r < k; r++)
        if (acc.a[r].coeffs != acc2.a[r].coeffs) return fail("trace and blindRotateMP21Ntt disagree");
    if (acc.b.coeffs != acc2.b.coeffs) return fail("trace and blindRotateMP21Ntt disagree");
    return 0;
}

// functionalBootstrappingMPNtt (yatfhe/src/bootstrapping.cpp:71-80), one call per
// ciphertext.  workers == 0: all on the calling thread (the external product fans its
// levels out on the reference thread pool, trgsw.cpp:753-759).  workers != 0: one pool
// task per ciphertext, so each pool worker runs whole bootstraps serially (the pool's
// size is fixed by YATFHE_THREADS or the affinity mask, multi_threading.cpp:22-38).
int ref_pbs(const int32_t* in, int count, const int64_t* v, int32_t* out, int workers) {
    auto& s = st();
    if (!s.bsk || !s.ksk) return fail("ref_pbs: keys not loaded");
    return guarded([&] {
        const auto& p = s.param;
        const int n = p.n, N = p.N;
        TorusPolynomial vp{N};
        toPoly(vp, v, N);
        auto one = [&](int c) {
            Tlwe x{n}, y{n};
            toTlwe(x, in + static_cast<size_t>(c) * (n + 1), n);
            functionalBootstrappingMPNtt(y, x, *s.bsk, *s.ksk, vp, p);
            fromTlwe(out + static_cast<size_t>(c) * (n + 1), y, n);
        };
        if (!workers) {
            for (int c = 0; c < count; c++) one(c);
            return;
        }
        std::vector<std::future<void>> fs;
        fs.reserve(count);
        for (int c = 0; c < count; c++) fs.emplace_back(ThreadPool::instance().enqueue(one, c));
        for (auto& f : fs) f.get();
    });
}

// ---------------------------------------------------------------- WWL+24 keys
// Key generation for the WWL+24 family on the calling thread's RNG stream 0: genTlweKey,
// genTrlweKey, then the per-i body of genBootstrappingKeyWWL24
// (yatfhe/src/bootstrapping.cpp:106-126) for i = 0..n-1 in order -- one
// symEncTrlweMultiSampleNtt of s_i g_lvl per level (yatfhe/src/trlwe.cpp:103-106) --,
// then its symEncTrlevWithKeyNtt of the RLWE secret (yatfhe/src/trlev.cpp:75-96) and
// genTlweKeySwitchingKey.  As for ref_keygen, the per-i calls run in order on one thread
// so that a seed gives one key.
int ref_keygen_wwl24(uint64_t seed) {
    if (!st().ready) return fail("ref_keygen_wwl24: ref_setup not called");
    return guarded([&] {
        auto& s = st();
        auto& p = s.param;
        (void)rng();
        yatfhe_oracle_set_seed(seed);
        rng = ChaCha20Rng();
        s.lweKey = std::make_unique<TlweKey>(p);
        s.trgswKey = std::make_unique<TrgswKey>(p);
        s.wwl = std::make_unique<BootstrappingKeyWWL24>(p, p.lApprox);
        s.ksk = std::make_unique<TlweKeySwitchingKey>(p);
        genTlweKey(*s.lweKey);
        genTrlweKey(s.trgswKey->trlweKey);
        for (int i = 0; i < s.wwl->n; i++) {
            TorusPolynomial muPoly{p.N};
            Trlwe tmp{p.k, p.N};
            for (int lvl = 0; lvl < s.wwl->bskDft[i].l; lvl++) {
                muPoly.coeffs[0] = s.lweKey->s[i] << (p.torusBits - (lvl + 1) * p.radixBits);
                symEncTrlweMultiSampleNtt(tmp, s.wwl->bskDft[i].cPrime[lvl], s.trgswKey->trlweKey, muPoly.coeffs);
            }
        }
        symEncTrlevWithKeyNtt(s.wwl->s2Dft, s.trgswKey->trlweKey, s.trgswKey->trlweKey.s, true, p);
        TlweKey ksTarget = *s.lweKey;
        genTlweKeySwitchingKey(*s.ksk, s.trgswKey->trlweKey, ksTarget, p);
    });
}

// The WWL+24 key's NTT-domain words: cprime = [i][lvl][poly][N] (poly = a[0..k-1] then b of
// bskDft[i].cPrime[lvl]), s2 = [lvl][poly][N] of s2Dft (yatfhe/include/yatfhe/bootstrapping.h:116-135).
int ref_export_wwl24(uint64_t* cprime, uint64_t* s2) {
    auto& s = st();
    if (!s.wwl) return fail("ref_export_wwl24: no WWL+24 key");
    const int k = s.param.k, N = s.param.N;
    auto put = [&](uint64_t*& o, const TrlweDft& t) {
        for (int poly = 0; poly <= k; poly++) {
            const NttPolynomial& P = poly < k ? t.a[poly] : t.b;
            std::memcpy(o, P.coeffs.data(), sizeof(uint64_t) * N);
            o += N;
        }
    };
    uint64_t* o = cprime;
    for (int i = 0; i < s.wwl->n; i++)
        for (const auto& t : s.wwl->bskDft[i].cPrime) put(o, t);
    o = s2;
    for (const auto& t : s.wwl->s2Dft.trlweDfts) put(o, t);
    return 0;
}

// The GINX rows the WWL+24 blind rotation builds for every key index before its external
// product: cRows[lvl] = switchTrlweToSecretEmbeddingNtt(cPrime[lvl], s2Dft)
// (yatfhe/src/trgsw.cpp:861-905, called from blindRotateWWL24Ntt, blind_rotate.cpp:1394-1397),
// written with cPrime[lvl] as [i][lvl][row][poly][N] -- the layout of ref_export_bsk_ntt.
int ref_wwl24_expand(uint64_t* out) {
    auto& s = st();
    if (!s.wwl) return fail("ref_wwl24_expand: no WWL+24 key");
    return guarded([&] {
        const auto& p = s.param;
        const int k = p.k, N = p.N;
        uint64_t* o = out;
        auto put = [&](const TrlweDft& t) {
            for (int poly = 0; poly <= k; poly++) {
                const NttPolynomial& P = poly < k ? t.a[poly] : t.b;
                std::memcpy(o, P.coeffs.data(), sizeof(uint64_t) * N);
                o += N;
            }
        };
        for (int i = 0; i < s.wwl->n; i++) {
            const auto& g = s.wwl->bskDft[i];
            for (int lvl = 0; lvl < g.l; lvl++) {
                std::vector<TrlweDft> rows(k, TrlweDft(k, N));
                switchTrlweToSecretEmbeddingNtt(rows, g.cPrime[lvl], s.wwl->s2Dft, p);
                for (int r = 0; r < k; r++) put(rows[r]);
                put(g.cPrime[lvl]);
            }
        }
    });
}

// serializeBskWWL24 / deserializeBskWWL24 (yatfhe/src/ya_serializer.cpp:220-246).
int ref_save_wwl24(const char* path) {
    if (!st().wwl) return fail("ref_save_wwl24: no WWL+24 key");
    return guarded([&] { serializeBskWWL24(*st().wwl, path); });
}

int ref_load_wwl24(const char* path) {
    if (!st().ready) return fail("ref_load_wwl24: ref_setup not called");
    return guarded([&] {
        auto& s = st();
        s.wwl = std::make_unique<BootstrappingKeyWWL24>();
        deserializeBskWWL24(*s.wwl, path, s.param.n);
    });
}

// functionalBootstrappingMPNtt's composition (yatfhe/src/bootstrapping.cpp:71-80) with the
// WWL+24 blind rotation blindRotateWWL24Ntt (yatfhe/src/blind_rotate.cpp:1383-1412) in
// place of blindRotateMP21Ntt, one ciphertext after the other.  acc0 (may be null) receives
// the accumulator of ciphertext 0 after the blind rotation, [a..., b].
int ref_pbs_wwl24(const int32_t* in, int count, const int64_t* v, int32_t* out, int64_t* acc0) {
    auto& s = st();
    if (!s.wwl || !s.ksk) return fail("ref_pbs_wwl24: keys not loaded");
    return guarded([&] {
        const auto& p = s.param;
        const int n = p.n, N = p.N, k = p.k;
        TorusPolynomial vp{N};
        toPoly(vp, v, N);
        for (int c = 0; c < count; c++) {
            Tlwe x{n}, y{n};
            toTlwe(x, in + static_cast<size_t>(c) * (n + 1), n);
            ScaledTlwe sc{2 * N, n};
            Trlwe acc{k, N};
            Tlwe big{s.ksk->nCurrKey};
            rescaleTlweToNewMod(sc, x);
            genNoiselessTrlweSample(acc, vp, sc);
            blindRotateWWL24Ntt(acc, *s.wwl, sc, p);
            if (c == 0 && acc0) {
                for (int r = 0; r < k; r++) fromPoly(acc0 + static_cast<size_t>(r) * N, acc.a[r], N);
                fromPoly(acc0 + static_cast<size_t>(k) * N, acc.b, N);
            }
            extractTlweFromTrlwe(big, acc, p.driftPhase);
            switchKeyForTlwe(y, *s.ksk, big, p);
            fromTlwe(out + static_cast<size_t>(c) * (n + 1), y, n);
        }
    });
}

// ---------------------------------------------------------------- lazy ("OURS") keys
// genBootstrappingKeyMPLazyPipeAlt (yatfhe/src/bootstrapping.cpp:322-339) with its per-i
// encryptTrgswMP calls (yatfhe/src/trgsw.cpp:18-34) run in order on the calling thread, after
// genTlweKey and genTrlweKey and before genTlweKeySwitchingKey, as ref_keygen_wwl24 does.
int ref_keygen_lazy(uint64_t seed) {
    if (!st().ready) return fail("ref_keygen_lazy: ref_setup not called");
    return guarded([&] {
        auto& s = st();
        auto& p = s.param;
        (void)rng();
        yatfhe_oracle_set_seed(seed);
        rng = ChaCha20Rng();
        s.lweKey = std::make_unique<TlweKey>(p);
        s.trgswKey = std::make_unique<TrgswKey>(p);
        s.lazy = std::make_unique<BootstrappingKeyMPLazyPipeAlt>(p, p.lApprox, true);
        s.ksk = std::make_unique<TlweKeySwitchingKey>(p);
        genTlweKey(*s.lweKey);
        genTrlweKey(s.trgswKey->trlweKey);
        for (int i = 0; i < s.lazy->n; i++) encryptTrgswMP(s.lazy->bskPrime[i], s.lweKey->s[i], *s.trgswKey, 0, p);
        symEncTrlevWithKeyNtt(s.lazy->s2Dft, s.trgswKey->trlweKey, s.trgswKey->trlweKey.s, true, p);
        TlweKey ksTarget = *s.lweKey;
        genTlweKeySwitchingKey(*s.ksk, s.trgswKey->trlweKey, ksTarget, p);
    });
}

// The lazy key's words: cprime = [i][lvl][poly][N] torus values (poly = a[0..k-1] then b of
// bskPrime[i].cPrime[lvl]), s2 = [lvl][poly][N] NTT-domain words of s2Dft.
int ref_export_lazy(int64_t* cprime, uint64_t* s2) {
    auto& s = st();
    if (!s.lazy) return fail("ref_export_lazy: no lazy key");
    const int k = s.param.k, N = s.param.N;
    int64_t* o = cprime;
    for (const auto& g : s.lazy->bskPrime)
        for (const auto& t : g.cPrime)
            for (int poly = 0; poly <= k; poly++) {
                fromPoly(o, poly < k ? t.a[poly] : t.b, N);
                o += N;
            }
    uint64_t* w = s2;
    for (const auto& t : s.lazy->s2Dft.trlweDfts)
        for (int poly = 0; poly <= k; poly++) {
            const NttPolynomial& P = poly < k ? t.a[poly] : t.b;
            std::memcpy(w, P.coeffs.data(), sizeof(uint64_t) * N);
            w += N;
        }
    return 0;
}

// serializeBskLazyPipeAlt / deserializeBskLazyPipeAlt (yatfhe/src/ya_serializer.cpp:445-481).
int ref_save_lazy(const char* path) {
    if (!st().lazy) return fail("ref_save_lazy: no lazy key");
    return guarded([&] { serializeBskLazyPipeAlt(*st().lazy, path); });
}

int ref_load_lazy(const char* path) {
    if (!st().ready) return fail("ref_load_lazy: ref_setup not called");
    return guarded([&] {
        auto& s = st();
        s.lazy = std::make_unique<BootstrappingKeyMPLazyPipeAlt>();
        deserializeBskLazyPipeAlt(*s.lazy, path, s.param.n);
    });
}

// functionalBootstrappingMPNtt's composition (yatfhe/src/bootstrapping.cpp:71-80) with
// blindRotateLazyPipeAltNtt (yatfhe/src/blind_rotate.cpp:995-999) in place of the MP21 blind
// rotation: prepareGdV once (yatfhe/src/trgsw.cpp:911-927), then per ciphertext the lazy blind
// rotation (which builds the accumulator from v itself), extraction and key switching.  acc0
// (may be null) receives ciphertext 0's accumulator after the blind rotation.
namespace {
int sweep_move = -1, sweep_units = 2;  // ref_pbs_lazy_sweep's split; -1: blindRotateLazyPipeAltNtt
bool lazy_no_first = false;            // ref_pbs_lazy_no_first: blindRotateLazyPipeAltNoFirstNtt
}

int ref_pbs_lazy(const int32_t* in, int count, const int64_t* v, int32_t* out, int64_t* acc0) {
    auto& s = st();
    if (!s.lazy || !s.ksk) return fail("ref_pbs_lazy: keys not loaded");
    return guarded([&] {
        const auto& p = s.param;
        const int n = p.n, N = p.N, k = p.k;
        TorusPolynomial vp{N};
        toPoly(vp, v, N);
        std::vector<NttPolynomial> gdV;
        prepareGdV(gdV, vp, p);
        for (int c = 0; c < count; c++) {
            Tlwe x{n}, y{n};
            toTlwe(x, in + static_cast<size_t>(c) * (n + 1), n);
            ScaledTlwe sc{2 * N, n};
            Trlwe acc{k, N};
            Tlwe big{s.ksk->nCurrKey};
            rescaleTlweToNewMod(sc, x);
            if (lazy_no_first)
                blindRotateLazyPipeAltNoFirstNtt(acc, *s.lazy, sc, vp, p);
            else if (sweep_move < 0)
                blindRotateLazyPipeAltNtt(acc, *s.lazy, sc, vp, gdV, p);
            else
                blindRotateLazyPipeAltNttSweep(acc, *s.lazy, sc, vp, gdV, sweep_move, sweep_units, p);
            if (c == 0 && acc0) {
                for (int r = 0; r < k; r++) fromPoly(acc0 + static_cast<size_t>(r) * N, acc.a[r], N);
                fromPoly(acc0 + static_cast<size_t>(k) * N, acc.b, N);
            }
            extractTlweFromTrlwe(big, acc, p.driftPhase);
            switchKeyForTlwe(y, *s.ksk, big, p);
            fromTlwe(out + static_cast<size_t>(c) * (n + 1), y, n);
        }
    });
}

// ---------------------------------------------------------------- group keys (BootstrappingKey)
// genTlweKey, genTrlweKey, genBootstrappingKey with param.group = group
// (yatfhe/src/bootstrapping.cpp:98-104: genBootstrappingKeyNormal for group 1,
// genBootstrappingKeyGroup :16-38 otherwise; both run in order on the calling thread), then
// genTlweKeySwitchingKey.
int ref_keygen_group(uint64_t seed, int group) {
    if (!st().ready) return fail("ref_keygen_group: ref_setup not called");
    return guarded([&] {
        auto& s = st();
        auto& p = s.param;
        p.group = group;
        (void)rng();
        yatfhe_oracle_set_seed(seed);
        rng = ChaCha20Rng();
        s.lweKey = std::make_unique<TlweKey>(p);
        s.trgswKey = std::make_unique<TrgswKey>(p);
        s.gbsk = std::make_unique<BootstrappingKey>(p);
        s.ksk = std::make_unique<TlweKeySwitchingKey>(p);
        genTlweKey(*s.lweKey);
        genTrlweKey(s.trgswKey->trlweKey);
        genBootstrappingKey(*s.gbsk, *s.trgswKey, *s.lweKey, p);
        TlweKey ksTarget = *s.lweKey;
        genTlweKeySwitchingKey(*s.ksk, s.trgswKey->trlweKey, ksTarget, p);
    });
}

// The group key's NTT-domain words, [j][lvl][row][poly][N] of bskDft[j].trlweDftSamples[lvl][row]
// (poly = a[0..k-1] then b), j < n / group * 2^group (n for group 1), lvl < param.l.
int ref_export_group(uint64_t* out) {
    auto& s = st();
    if (!s.gbsk) return fail("ref_export_group: no group key");
    const int k = s.param.k, N = s.param.N;
    uint64_t* o = out;
    for (const auto& g : s.gbsk->bskDft)
        for (const auto& lv : g.trlweDftSamples)
            for (const auto& t : lv)
                for (int poly = 0; poly <= k; poly++) {
                    const NttPolynomial& P = poly < k ? t.a[poly] : t.b;
                    std::memcpy(o, P.coeffs.data(), sizeof(uint64_t) * N);
                    o += N;
                }
    return 0;
}

// functionalBootstrappingNtt (yatfhe/src/bootstrapping.cpp:60-68) on the group key, one
// ciphertext after the other: rescaleTlweToNewMod, genNoiselessTrlweSample, blindRotateNtt
// (yatfhe/src/blind_rotate.cpp:549-560: blindRotateNormalNtt, blindRotateGroup2Ntt or
// blindRotateGroup3Ntt by the key's group), extraction, key switching.  acc0 (may be null)
// receives ciphertext 0's accumulator after the blind rotation.
int ref_pbs_group(const int32_t* in, int count, const int64_t* v, int32_t* out, int64_t* acc0) {
    auto& s = st();
    if (!s.gbsk || !s.ksk) return fail("ref_pbs_group: keys not loaded");
    return guarded([&] {
        YatfheParameters p = s.param;
        p.group = s.gbsk->group;
        const int n = p.n, N = p.N, k = p.k;
        TorusPolynomial vp{N};
        toPoly(vp, v, N);
        for (int c = 0; c < count; c++) {
            Tlwe x{n}, y{n};
            toTlwe(x, in + static_cast<size_t>(c) * (n + 1), n);
            ScaledTlwe sc{2 * N, n};
            Trlwe acc{k, N};
            Tlwe big{s.ksk->nCurrKey};
            rescaleTlweToNewMod(sc, x);
            genNoiselessTrlweSample(acc, vp, sc);
            blindRotateNtt(acc, s.gbsk->bskDft, sc, p);
            if (c == 0 && acc0) {
                for (int r = 0; r < k; r++) fromPoly(acc0 + static_cast<size_t>(r) * N, acc.a[r], N);
                fromPoly(acc0 + static_cast<size_t>(k) * N, acc.b, N);
            }
            extractTlweFromTrlwe(big, acc, p.driftPhase);
            switchKeyForTlwe(y, *s.ksk, big, p);
            fromTlwe(out + static_cast<size_t>(c) * (n + 1), y, n);
        }
    });
}

// ref_pbs_lazy with blindRotateLazyPipeAltNttSweep (yatfhe/src/blind_rotate.cpp:1001-1135) and
// the given split of its pipeline (moveNtt digit levels transformed in stageA, unitsA workers).
int ref_pbs_lazy_sweep(const int32_t* in, int count, const int64_t* v, int32_t* out, int move_ntt, int units_a) {
    sweep_move = move_ntt;
    sweep_units = units_a;
    const int rc = ref_pbs_lazy(in, count, v, out, nullptr);
    sweep_move = -1;
    return rc;
}

// ref_pbs_lazy with blindRotateLazyPipeAltNoFirstNtt (yatfhe/src/blind_rotate.cpp:1137-1267)
// in place of blindRotateLazyPipeAltNtt.
int ref_pbs_lazy_no_first(const int32_t* in, int count, const int64_t* v, int32_t* out, int64_t* acc0) {
    lazy_no_first = true;
    const int rc = ref_pbs_lazy(in, count, v, out, acc0);
    lazy_no_first = false;
    return rc;
}

int ref_pool_size(void) { return static_cast<int>(ThreadPool::usableConcurrency()); }

// ---------------------------------------------------------------- approximate CRT (ApproxCRT)
// The setting of the reference's BLIND_ROT_APPROX_CRT(_NTT) tests (google_tests/blindrot_test.cpp:
// 505-640): the torus is Q_CRT = 251 241 239 233 (param.q = Q_CRT), the accumulator is kept as
// d = 4 Trlwe8 residue samples, the key is BootstrappingKeyCRT (yatfhe/include/yatfhe/
// bootstrapping.h:351-361).  param.l is set to param.dh (2): encryptTrgswApproxCRT adds
// param.w[lvl] for every level of a Trgsw{param} (yatfhe/src/trgsw.cpp:248-263) and w has dh
// entries, while decompTrgswMcrt keeps the first dh levels (yatfhe/src/trgsw.cpp:334-360).

static std::unique_ptr<BootstrappingKeyCRT> crt_key;

int ref_crt_setup(int n, int N, int rlwe_noise_b, int torus_base) {
    return guarded([&] {
        auto& s = st();
        s.param = YatfheParameters{};
        auto& q = s.param;
        q.q = Q_CRT;
        q.n = n;
        q.N = N;
        q.l = q.dh;
        q.rlweNoiseB = rlwe_noise_b;
        q.torusBase = torus_base;
        initYatfhe(q);
        s.lweKey.reset();
        s.trgswKey.reset();
        s.bsk.reset();
        s.wwl.reset();
        s.lazy.reset();
        s.gbsk.reset();
        s.ksk.reset();
        crt_key.reset();
        s.ready = true;
    });
}

// genTlweKey, genTrlweKey, then the per-i body of genBootstrappingKeyApproxCrt
// (yatfhe/src/bootstrapping.cpp:425-440: encryptTrgswApproxCRT, decompTrgswMcrt, the NTT24 of
// every residue Trgsw8) for i = 0..n-1 in order on one RNG stream.
int ref_crt_keygen(uint64_t seed) {
    if (!st().ready) return fail("ref_crt_keygen: ref_crt_setup not called");
    return guarded([&] {
        auto& s = st();
        auto& p = s.param;
        (void)rng();
        yatfhe_oracle_set_seed(seed);
        rng = ChaCha20Rng();
        s.lweKey = std::make_unique<TlweKey>(p);
        s.trgswKey = std::make_unique<TrgswKey>(p);
        crt_key = std::make_unique<BootstrappingKeyCRT>(p);
        genTlweKey(*s.lweKey);
        genTrlweKey(s.trgswKey->trlweKey);
        for (int i = 0; i < p.n; i++) {
            Trgsw tmp{p};
            encryptTrgswApproxCRT(tmp, p, *s.trgswKey, s.lweKey->s[i]);
            decompTrgswMcrt(crt_key->bsk8[i], tmp, p);
            for (int d = 0; d < p.d; d++) NttNative24::applyNttForRgsw(crt_key->bskCRT[i][d], crt_key->bsk8[i][d]);
        }
    });
}

// bsk8 as int8 [n][d][dh][k+1 rows][k+1 polys: a_0 .. a_{k-1}, b][N].
int ref_crt_export_bsk8(int8_t* out) {
    if (!crt_key) return fail("ref_crt_export_bsk8: no key");
    const auto& p = st().param;
    size_t o = 0;
    for (int i = 0; i < p.n; i++)
        for (int d = 0; d < p.d; d++)
            for (int l = 0; l < p.dh; l++)
                for (int r = 0; r <= p.k; r++) {
                    const auto& t = crt_key->bsk8[i][d].trlweSamples[l][r];
                    for (int c = 0; c <= p.k; c++) {
                        const auto& poly = c < p.k ? t.a[c] : t.b;
                        std::memcpy(out + o, poly.coeffs.data(), p.N);
                        o += p.N;
                    }
                }
    return 0;
}

// The other direction, for keys made elsewhere (the NTT24 forms are recomputed).
int ref_crt_import_bsk8(const int8_t* in) {
    if (!st().ready) return fail("ref_crt_import_bsk8: ref_crt_setup not called");
    return guarded([&] {
        const auto& p = st().param;
        crt_key = std::make_unique<BootstrappingKeyCRT>(p);
        size_t o = 0;
        for (int i = 0; i < p.n; i++)
            for (int d = 0; d < p.d; d++) {
                for (int l = 0; l < p.dh; l++)
                    for (int r = 0; r <= p.k; r++) {
                        auto& t = crt_key->bsk8[i][d].trlweSamples[l][r];
                        for (int c = 0; c <= p.k; c++) {
                            auto& poly = c < p.k ? t.a[c] : t.b;
                            std::memcpy(poly.coeffs.data(), in + o, p.N);
                            o += p.N;
                        }
                    }
                NttNative24::applyNttForRgsw(crt_key->bskCRT[i][d], crt_key->bsk8[i][d]);
            }
    });
}

// symEncTrlweMultiSample (yatfhe/src/trlwe.cpp:98-101) of plain [N] (messages mod torus_base,
// modSwitchToTorus32 as the reference's test does): out [k+1][N] torus values (a, then b).
int ref_crt_encrypt(const int32_t* plain, int64_t* out) {
    if (!st().trgswKey) return fail("ref_crt_encrypt: no key");
    return guarded([&] {
        const auto& p = st().param;
        std::vector<Torus> mu(p.N);
        for (int j = 0; j < p.N; j++) mu[j] = modSwitchToTorus32(plain[j], p.torusBase);
        Trlwe t{p.k, p.N};
        symEncTrlweMultiSample(t, st().trgswKey->trlweKey, mu);
        for (int c = 0; c < p.k; c++) fromPoly(out + (size_t)c * p.N, t.a[c], p.N);
        fromPoly(out + (size_t)p.k * p.N, t.b, p.N);
    });
}

// symDecTrlweToInt (yatfhe/src/trlwe.cpp:131-138).
int ref_crt_decrypt(const int64_t* in, int32_t* out) {
    if (!st().trgswKey) return fail("ref_crt_decrypt: no key");
    return guarded([&] {
        const auto& p = st().param;
        Trlwe t{p.k, p.N};
        for (int c = 0; c < p.k; c++) toPoly(t.a[c], in + (size_t)c * p.N, p.N);
        toPoly(t.b, in + (size_t)p.k * p.N, p.N);
        IntPolynomial dec{p.N};
        symDecTrlweToInt(dec, t, st().trgswKey->trlweKey, p.torusBase);
        for (int j = 0; j < p.N; j++) out[j] = static_cast<int32_t>(dec.coeffs[j]);
    });
}

// The reference test's sequence around the blind rotation: decompTrlweMcrt, then
// blindRotateApproxCRTNtt (ntt != 0) or blindRotateApproxCRT (yatfhe/src/blind_rotate.cpp:
// 563-589), trlweMcrtToCrt and recompTrlweCrt (yatfhe/include/yatfhe/trlwe.h:333-440).
// in/out: [k+1][N] torus values; rot [n]: the rotation amounts a_i; mcrt (if not null):
// the d residue samples after the rotation, int8 [d][k+1][N].
int ref_crt_blind_rotate(const int64_t* in, const int32_t* rot, int ntt, int64_t* out, int8_t* mcrt) {
    if (!crt_key) return fail("ref_crt_blind_rotate: no key");
    return guarded([&] {
        const auto& p = st().param;
        Trlwe t{p.k, p.N};
        for (int c = 0; c < p.k; c++) toPoly(t.a[c], in + (size_t)c * p.N, p.N);
        toPoly(t.b, in + (size_t)p.k * p.N, p.N);
        ScaledTlwe s{p.N * 2, p.n};
        for (int i = 0; i < p.n; i++) s.a[i] = rot[i];
        std::vector<Trlwe8> acc(p.d, Trlwe8{p.k, p.N});
        decompTrlweMcrt(acc, t, p);
        if (ntt) blindRotateApproxCRTNtt(acc, crt_key->bskCRT, s, p);
        else blindRotateApproxCRT(acc, crt_key->bsk8, s, p);
        if (mcrt)
            for (int d = 0; d < p.d; d++)
                for (int c = 0; c <= p.k; c++) {
                    const auto& poly = c < p.k ? acc[d].a[c] : acc[d].b;
                    std::memcpy(mcrt + ((size_t)d * (p.k + 1) + c) * p.N, poly.coeffs.data(), p.N);
                }
        trlweMcrtToCrt(acc, p);
        Trlwe r{p.k, p.N};
        recompTrlweCrt(r, acc, p);
        for (int c = 0; c < p.k; c++) fromPoly(out + (size_t)c * p.N, r.a[c], p.N);
        fromPoly(out + (size_t)p.k * p.N, r.b, p.N);
    });
}

}  // extern "C"
