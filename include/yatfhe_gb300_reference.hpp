// yatfhe_gb300_reference.hpp -- the reference library's own C++ bootstrap signatures,
// implemented on the GB300 C ABI (yatfhe_gb300.h).
//
// For programs built against the yatfhe reference headers (yatfhe/include): include this
// header after them and call yatfhe_gb300::functionalBootstrappingMPNtt & co. with the
// reference's own types; a `using namespace yatfhe_gb300;` or a qualified call swaps the
// CPU implementation for the GPU one without touching the surrounding code.  Keys are
// converted and uploaded on first use and cached per key object (address) together with a
// fingerprint (sizes and a few dozen words sampled across the key): a different key built
// later at the same address is recognised and uploaded again.  A key changed in place is
// only recognised if a sampled word changed: call yatfhe_gb300::forgetKeys() after
// mutating a key, and to release the device copies.  Failures throw the
// exception types the reference throws (std::invalid_argument for bad shapes, and
// std::runtime_error otherwise).
//
// Replaced entry points (reference paths relative to its project):
//   functionalBootstrappingMPNtt   yatfhe/include/yatfhe/bootstrapping.h:369-370
//   blindRotateMP21Ntt             yatfhe/include/yatfhe/blind_rotate.h:69
//   blindRotateJP22Ntt             yatfhe/include/yatfhe/blind_rotate.h:65 (binary keys)
//   blindRotateWWL24Ntt            yatfhe/include/yatfhe/blind_rotate.h:61
//   blindRotateLazyPipeAltNtt      yatfhe/include/yatfhe/blind_rotate.h:44-45
//   blindRotateLazyPipeAltNttSweep yatfhe/include/yatfhe/blind_rotate.h:48-50
//   blindRotateLazyPipeAltInitNtt  yatfhe/include/yatfhe/blind_rotate.h:56-57
//   blindRotateLazyPipeAltNoFirstNtt yatfhe/include/yatfhe/blind_rotate.h:53
//   blindRotateNtt                 yatfhe/include/yatfhe/blind_rotate.h:13 (groups 1-3)
//   functionalBootstrappingNtt     yatfhe/include/yatfhe/bootstrapping.h:366-367
//   switchKeyForTlwe               yatfhe/include/yatfhe/keyswitching.h:48
//   blindRotateApproxCRTNtt        yatfhe/include/yatfhe/blind_rotate.h:18-19
// plus a batched form of the first, which the reference does not have.
#ifndef YATFHE_GB300_REFERENCE_HPP
#define YATFHE_GB300_REFERENCE_HPP

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "yatfhe_gb300.h"
#include "yautil/ya_serializer.h"  // deserializeBskLazyPipeAlt, for blindRotateLazyPipeAltInitNtt
#include "yatfhe/ntt24.h"          // NttNative24::applyIntt, for blindRotateApproxCRTNtt's key

namespace yatfhe_gb300 {

namespace detail {

inline void check(int rc) {
    if (rc == YG_OK) return;
    const std::string msg = yg_last_error();
    if (rc == YG_ERR_INVALID) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

inline void cuda(cudaError_t e) {
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

struct CachedKey {
    yg_key* key = nullptr;
    uint64_t fp = 0;             // fingerprint of the key object it was made from
    const void* ksk = nullptr;   // key-switching key attached to it, and its fingerprint
    uint64_t ksk_fp = 0;
};

struct CachedCrtKey {
    yg_crt_key* key = nullptr;
    uint64_t fp = 0;
};

struct Registry {
    std::mutex mu;
    std::map<std::tuple<int, int, int, int, int, int, int, int>, yg_ctx*> ctxs;
    std::map<const void*, CachedKey> keys;  // key object address -> device key
    std::map<const void*, CachedCrtKey> crt_keys;  // BootstrappingKeyCRT::bskCRT address -> device key

    ~Registry() {
        for (auto& k : keys) yg_key_destroy(k.second.key);
        for (auto& k : crt_keys) yg_crt_key_destroy(k.second.key);
        for (auto& c : ctxs) yg_ctx_destroy(c.second);
    }
};

inline Registry& reg() {
    static Registry r;
    return r;
}

inline uint64_t mix(uint64_t h, uint64_t v) { return (h ^ (v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2))) * 0x100000001b3ULL; }

template <typename P>
inline uint64_t mix_poly(uint64_t h, const P& poly) {
    const size_t m = poly.coeffs.size();
    h = mix(h, m);
    if (m)
        for (size_t j : {size_t(0), m / 3, m / 2, m - 1}) h = mix(h, static_cast<uint64_t>(poly.coeffs[j]));
    return h;
}

// the first, middle and last entries of a non-empty vector
template <typename V>
inline std::vector<size_t> probes(const V& v) {
    return v.empty() ? std::vector<size_t>{} : std::vector<size_t>{0, v.size() / 2, v.size() - 1};
}

template <typename T>
inline uint64_t mix_trlwe(uint64_t h, const T& t) {
    for (const auto& a : t.a) h = mix_poly(h, a);
    return mix_poly(h, t.b);
}

inline uint64_t fingerprint(const std::vector<std::vector<TrgswMPDft>>& bskDft) {
    uint64_t h = mix(0, bskDft.size());
    for (size_t i : probes(bskDft)) {
        const TrgswMPDft& t = bskDft[i][0];
        h = mix(h, static_cast<uint64_t>(t.l));
        for (size_t lvl : probes(t.cPrime)) {
            h = mix_trlwe(h, t.cPrime[lvl]);
            if (lvl < t.c.size())
                for (const auto& r : t.c[lvl]) h = mix_trlwe(h, r);
        }
    }
    return h;
}

inline uint64_t fingerprint(const TlweKeySwitchingKey& ksk) {
    uint64_t h = mix(1, ksk.decomposedKsk.size());
    for (size_t i : probes(ksk.decomposedKsk))
        for (size_t j : probes(ksk.decomposedKsk[i])) {
            const Tlwe& t = ksk.decomposedKsk[i][j];
            for (size_t e : probes(t.a)) h = mix(h, static_cast<uint64_t>(t.a[e]));
            h = mix(h, static_cast<uint64_t>(t.b));
        }
    return h;
}

// The cached device key of the object at `addr` if its fingerprint still matches; a stale
// entry (another key now at that address) is released.
inline CachedKey* cached(const void* addr, uint64_t fp) {
    auto& r = reg();
    auto it = r.keys.find(addr);
    if (it == r.keys.end()) return nullptr;
    if (it->second.fp == fp) return &it->second;
    yg_key_destroy(it->second.key);
    r.keys.erase(it);
    return nullptr;
}

inline void attach_ksk(CachedKey& e, const TlweKeySwitchingKey& ksk) {
    const uint64_t fp = fingerprint(ksk);
    if (e.ksk == &ksk && e.ksk_fp == fp) return;
    std::vector<int32_t> flat;
    for (const auto& row : ksk.decomposedKsk)
        for (const auto& t : row) {
            for (auto a : t.a) flat.push_back(static_cast<int32_t>(a));
            flat.push_back(static_cast<int32_t>(t.b));
        }
    check(yg_key_set_ksk(e.key, flat.data()));
    e.ksk = &ksk;
    e.ksk_fp = fp;
}

inline yg_params params_of(const YatfheParameters& p, int levels) {
    return yg_params{p.n, p.N, p.k, p.radixBits, levels, p.ksRadixBits, p.ksLevel, p.torusBits};
}

inline yg_ctx* context(const yg_params& q) {
    auto& r = reg();
    auto key = std::make_tuple(q.n, q.N, q.k, q.radix_bits, q.l_approx, q.ks_radix_bits, q.ks_level, q.torus_bits);
    auto it = r.ctxs.find(key);
    if (it != r.ctxs.end()) return it->second;
    yg_ctx* c = nullptr;
    check(yg_ctx_create(&q, 0, &c));
    r.ctxs[key] = c;
    return c;
}

// BootstrappingKeyMP::bskDft -> [n][l][k+1][k+1][N] words.
inline std::vector<uint64_t> flatten(const std::vector<std::vector<TrgswMPDft>>& bskDft, int k, int N) {
    std::vector<uint64_t> w;
    for (const auto& g : bskDft) {
        const TrgswMPDft& t = g[0];
        for (int lvl = 0; lvl < t.l; lvl++)
            for (int row = 0; row <= k; row++) {
                const TrlweDft& r = row < k ? t.c[lvl][row] : t.cPrime[lvl];
                for (int poly = 0; poly <= k; poly++) {
                    const auto& P = poly < k ? r.a[poly] : r.b;
                    w.insert(w.end(), P.coeffs.begin(), P.coeffs.begin() + N);
                }
            }
    }
    return w;
}

inline yg_key* device_key(yg_ctx* c, const std::vector<std::vector<TrgswMPDft>>& bskDft, const TlweKeySwitchingKey* ksk,
                          int k, int N) {
    const uint64_t fp = fingerprint(bskDft);
    CachedKey* e = cached(&bskDft, fp);
    if (!e) {
        const auto w = flatten(bskDft, k, N);
        yg_key* key = nullptr;
        check(yg_key_upload_bsk_ntt(c, w.data(), &key));
        e = &(reg().keys[&bskDft] = CachedKey{key, fp, nullptr, 0});
    }
    if (ksk) attach_ksk(*e, *ksk);
    return e->key;
}

// BootstrappingKeyWWL24 (yatfhe/include/yatfhe/bootstrapping.h:116-135) -> device key: the
// cPrime rows [n][l][k+1][N] and the s2 key [levels][k+1][N]; the GPU derives the GINX rows.
inline yg_key* device_key_wwl24(yg_ctx* c, const BootstrappingKeyWWL24& bsk, int k, int N) {
    uint64_t fp = mix(2, bsk.bskDft.size());
    for (size_t i : probes(bsk.bskDft))
        for (size_t lvl : probes(bsk.bskDft[i].cPrime)) fp = mix_trlwe(fp, bsk.bskDft[i].cPrime[lvl]);
    for (size_t lvl : probes(bsk.s2Dft.trlweDfts)) fp = mix_trlwe(fp, bsk.s2Dft.trlweDfts[lvl]);
    if (CachedKey* e = cached(&bsk, fp)) return e->key;
    std::vector<uint64_t> cprime, s2;
    auto put = [&](std::vector<uint64_t>& w, const TrlweDft& t) {
        for (int poly = 0; poly <= k; poly++) {
            const auto& P = poly < k ? t.a[poly] : t.b;
            w.insert(w.end(), P.coeffs.begin(), P.coeffs.begin() + N);
        }
    };
    for (const auto& g : bsk.bskDft)
        for (const auto& t : g.cPrime) put(cprime, t);
    for (const auto& t : bsk.s2Dft.trlweDfts) put(s2, t);
    yg_key* key = nullptr;
    check(yg_key_upload_wwl24_ntt(c, cprime.data(), s2.data(), static_cast<int>(bsk.s2Dft.trlweDfts.size()), &key));
    reg().keys[&bsk] = CachedKey{key, fp, nullptr, 0};
    return key;
}

// BootstrappingKeyMPLazyPipeAlt (yatfhe/include/yatfhe/bootstrapping.h:284-307) -> device key:
// the half rows bskPrime[i].cPrime [n][l][k+1][N] as torus values and the s2 key
// [levels][k+1][N]; the device keeps both as they are.
inline yg_key* device_key_lazy(yg_ctx* c, const BootstrappingKeyMPLazyPipeAlt& bsk, int k, int N) {
    uint64_t fp = mix(3, bsk.bskPrime.size());
    for (size_t i : probes(bsk.bskPrime))
        for (size_t lvl : probes(bsk.bskPrime[i].cPrime)) fp = mix_trlwe(fp, bsk.bskPrime[i].cPrime[lvl]);
    for (size_t lvl : probes(bsk.s2Dft.trlweDfts)) fp = mix_trlwe(fp, bsk.s2Dft.trlweDfts[lvl]);
    if (CachedKey* e = cached(&bsk, fp)) return e->key;
    std::vector<int64_t> cprime;
    std::vector<uint64_t> s2;
    for (const auto& g : bsk.bskPrime)
        for (const auto& t : g.cPrime)
            for (int poly = 0; poly <= k; poly++) {
                const auto& P = poly < k ? t.a[poly] : t.b;
                for (int j = 0; j < N; j++) cprime.push_back(static_cast<int64_t>(P.coeffs[j]));
            }
    for (const auto& t : bsk.s2Dft.trlweDfts)
        for (int poly = 0; poly <= k; poly++) {
            const auto& P = poly < k ? t.a[poly] : t.b;
            s2.insert(s2.end(), P.coeffs.begin(), P.coeffs.begin() + N);
        }
    yg_key* key = nullptr;
    check(yg_key_upload_lazy(c, cprime.data(), s2.data(), static_cast<int>(bsk.s2Dft.trlweDfts.size()), &key));
    reg().keys[&bsk] = CachedKey{key, fp, nullptr, 0};
    return key;
}

// BootstrappingKey (yatfhe/include/yatfhe/bootstrapping.h:16-45) -> device key: the TrgswDft
// words of every key, [keys][l][k+1][k+1][N], with the key's group; the key-switching key
// attached when given.
inline yg_key* device_key_group(yg_ctx* c, const std::vector<TrgswDft>& bskDft, int group,
                                const TlweKeySwitchingKey* ksk, int k, int N) {
    uint64_t fp = mix(mix(4, static_cast<uint64_t>(group)), bskDft.size());
    for (size_t i : probes(bskDft))
        for (size_t lvl : probes(bskDft[i].trlweDftSamples))
            for (const auto& t : bskDft[i].trlweDftSamples[lvl]) fp = mix_trlwe(fp, t);
    CachedKey* e = cached(&bskDft, fp);
    if (!e) {
        yg_key* key = nullptr;
        std::vector<uint64_t> words;
        for (const auto& g : bskDft)
            for (const auto& lv : g.trlweDftSamples)
                for (const auto& t : lv)
                    for (int poly = 0; poly <= k; poly++) {
                        const auto& P = poly < k ? t.a[poly] : t.b;
                        words.insert(words.end(), P.coeffs.begin(), P.coeffs.begin() + N);
                    }
        const int levels = bskDft.empty() ? 0 : bskDft[0].l;
        check(yg_key_upload_group(c, words.data(), group, levels, &key));
        e = &(reg().keys[&bskDft] = CachedKey{key, fp, nullptr, 0});
    }
    if (ksk) attach_ksk(*e, *ksk);
    return e->key;
}

template <typename T>
struct DeviceBuf {
    T* p = nullptr;
    explicit DeviceBuf(size_t n) { cuda(cudaMalloc(&p, n * sizeof(T))); }
    ~DeviceBuf() { cudaFree(p); }
};

}  // namespace detail

inline void forgetKeys() {
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    for (auto& k : r.keys) yg_key_destroy(k.second.key);
    r.keys.clear();
    for (auto& k : r.crt_keys) yg_crt_key_destroy(k.second.key);
    r.crt_keys.clear();
}

// Batched functionalBootstrappingMPNtt: out[i] = PBS(in[i]) under one key, one launch.
inline void functionalBootstrappingMPNttBatch(std::vector<Tlwe>& out, const std::vector<Tlwe>& in,
                                              const BootstrappingKeyMP& bsk, const TlweKeySwitchingKey& ksk,
                                              const TorusPolynomial& v, const YatfheParameters& param) {
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    const int levels = bsk.bskDft.empty() ? param.lApprox : bsk.bskDft[0][0].l;
    yg_ctx* c = detail::context(detail::params_of(param, levels));
    yg_key* key = detail::device_key(c, bsk.bskDft, &ksk, param.k, param.N);
    const int n = param.n, count = static_cast<int>(in.size());
    std::vector<int32_t> h_in(static_cast<size_t>(count) * (n + 1)), h_out(h_in.size());
    for (int i = 0; i < count; i++) {
        for (int j = 0; j < n; j++) h_in[static_cast<size_t>(i) * (n + 1) + j] = static_cast<int32_t>(in[i].a[j]);
        h_in[static_cast<size_t>(i) * (n + 1) + n] = static_cast<int32_t>(in[i].b);
    }
    std::vector<int64_t> lut(v.coeffs.begin(), v.coeffs.end());
    detail::check(yg_pbs_host(c, key, h_in.data(), h_out.data(), count, lut.data(), nullptr));
    out.resize(count, Tlwe(n));
    for (int i = 0; i < count; i++) {
        for (int j = 0; j < n; j++) out[i].a[j] = static_cast<LweTorus>(h_out[static_cast<size_t>(i) * (n + 1) + j]);
        out[i].b = static_cast<LweTorus>(h_out[static_cast<size_t>(i) * (n + 1) + n]);
    }
}

inline void functionalBootstrappingMPNtt(Tlwe& out, const Tlwe& input, const BootstrappingKeyMP& bsk,
                                         const TlweKeySwitchingKey& ksk, const TorusPolynomial& v,
                                         const YatfheParameters& param) {
    std::vector<Tlwe> o, i{input};
    functionalBootstrappingMPNttBatch(o, i, bsk, ksk, v, param);
    out = o[0];
}

namespace detail {

// accum (already genNoiselessTrlweSample'd) rotated in place under `key`.
inline void rotate_accumulator(yg_ctx* c, yg_key* key, Trlwe& accum, const ScaledTlwe& input,
                               const YatfheParameters& param) {
    const int n = param.n, N = param.N, k = param.k;
    std::vector<int32_t> a(input.a.begin(), input.a.end());
    std::vector<int64_t> acc(static_cast<size_t>(k + 1) * N);
    for (int p = 0; p < k; p++)
        for (int j = 0; j < N; j++) acc[static_cast<size_t>(p) * N + j] = accum.a[p].coeffs[j];
    for (int j = 0; j < N; j++) acc[static_cast<size_t>(k) * N + j] = accum.b.coeffs[j];
    DeviceBuf<int32_t> d_a(n);
    DeviceBuf<int64_t> d_acc(acc.size());
    cuda(cudaMemcpy(d_a.p, a.data(), a.size() * 4, cudaMemcpyHostToDevice));
    cuda(cudaMemcpy(d_acc.p, acc.data(), acc.size() * 8, cudaMemcpyHostToDevice));
    check(yg_blind_rotate_acc(c, key, d_a.p, d_acc.p, 1, nullptr));
    cuda(cudaMemcpy(acc.data(), d_acc.p, acc.size() * 8, cudaMemcpyDeviceToHost));
    for (int p = 0; p < k; p++)
        for (int j = 0; j < N; j++) accum.a[p].coeffs[j] = static_cast<Torus>(acc[static_cast<size_t>(p) * N + j]);
    for (int j = 0; j < N; j++) accum.b.coeffs[j] = static_cast<Torus>(acc[static_cast<size_t>(k) * N + j]);
}

}  // namespace detail

// blindRotateMP21Ntt: accum (already genNoiselessTrlweSample'd) is rotated in place.
inline void blindRotateMP21Ntt(Trlwe& accum, const std::vector<std::vector<TrgswMPDft>>& bskDft,
                               const ScaledTlwe& input, const YatfheParameters& param) {
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    yg_ctx* c = detail::context(detail::params_of(param, bskDft[0][0].l));
    yg_key* key = detail::device_key(c, bskDft, nullptr, param.k, param.N);
    detail::rotate_accumulator(c, key, accum, input, param);
}

// blindRotateWWL24Ntt: the same rotation on a WWL+24 key (its GINX rows derived once, on the GPU).
inline void blindRotateWWL24Ntt(Trlwe& accum, const BootstrappingKeyWWL24& bsk, const ScaledTlwe& input,
                                const YatfheParameters& param) {
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    const int levels = bsk.bskDft.empty() ? param.lApprox : bsk.bskDft[0].l;
    yg_ctx* c = detail::context(detail::params_of(param, levels));
    yg_key* key = detail::device_key_wwl24(c, bsk, param.k, param.N);
    detail::rotate_accumulator(c, key, accum, input, param);
}

// blindRotateLazyPipeAltNtt: accum receives the lazy blind rotation of input with test
// polynomial v (the rotation builds its accumulator from v, as the reference's does).
// gdVntt, prepareGdV(v) in the reference, is derived from v on the GPU and not read.
inline void blindRotateLazyPipeAltNtt(Trlwe& accum, const BootstrappingKeyMPLazyPipeAlt& bsk, const ScaledTlwe& input,
                                      const TorusPolynomial& v, const std::vector<NttPolynomial>& gdVntt,
                                      const YatfheParameters& param) {
    (void)gdVntt;
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    const int n = param.n, N = param.N, k = param.k;
    const int levels = bsk.bskPrime.empty() ? param.lApprox : bsk.bskPrime[0].l;
    yg_ctx* c = detail::context(detail::params_of(param, levels));
    yg_key* key = detail::device_key_lazy(c, bsk, k, N);
    // the mod-2N input as 32-bit words that switch back to the same values: x 2^(32 - log2(2N))
    int sh = 32;
    for (int m = 2 * N; m > 1; m >>= 1) sh--;
    std::vector<int32_t> words(static_cast<size_t>(n) + 1);
    for (int i = 0; i < n; i++) words[i] = static_cast<int32_t>(static_cast<uint32_t>(input.a[i]) << sh);
    words[n] = static_cast<int32_t>(static_cast<uint32_t>(input.b) << sh);
    std::vector<int64_t> lut(N), acc(static_cast<size_t>(k + 1) * N);
    for (int j = 0; j < N; j++) lut[j] = static_cast<int64_t>(v.coeffs[j]);
    detail::DeviceBuf<int32_t> d_in(words.size());
    detail::DeviceBuf<int64_t> d_lut(lut.size());
    detail::DeviceBuf<int64_t> d_acc(acc.size());
    detail::cuda(cudaMemcpy(d_in.p, words.data(), words.size() * 4, cudaMemcpyHostToDevice));
    detail::cuda(cudaMemcpy(d_lut.p, lut.data(), lut.size() * 8, cudaMemcpyHostToDevice));
    detail::check(yg_blind_rotate(c, key, d_in.p, d_lut.p, d_acc.p, 1, n, nullptr));
    detail::cuda(cudaMemcpy(acc.data(), d_acc.p, acc.size() * 8, cudaMemcpyDeviceToHost));
    for (int p = 0; p < k; p++)
        for (int j = 0; j < N; j++) accum.a[p].coeffs[j] = static_cast<Torus>(acc[static_cast<size_t>(p) * N + j]);
    for (int j = 0; j < N; j++) accum.b.coeffs[j] = static_cast<Torus>(acc[static_cast<size_t>(k) * N + j]);
}

// blindRotateNtt: the group-g blind rotation (param.group selects blindRotateNormalNtt,
// blindRotateGroup2Ntt or blindRotateGroup3Ntt, as in the reference) of accum, already
// genNoiselessTrlweSample'd, in place.
inline void blindRotateNtt(Trlwe& accum, const std::vector<TrgswDft>& bskDft, const ScaledTlwe& input,
                           const YatfheParameters& param) {
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    yg_ctx* c = detail::context(detail::params_of(param, param.lApprox));
    yg_key* key = detail::device_key_group(c, bskDft, param.group, nullptr, param.k, param.N);
    detail::rotate_accumulator(c, key, accum, input, param);
}

// functionalBootstrappingNtt: the bootstrap on a group key (rescale, noiseless sample,
// blindRotateNtt, extraction, key switching), one ciphertext.
inline void functionalBootstrappingNtt(Tlwe& out, const Tlwe& input, const BootstrappingKey& bsk,
                                       const TlweKeySwitchingKey& ksk, const TorusPolynomial& v,
                                       const YatfheParameters& param) {
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    const int n = param.n, N = param.N;
    yg_ctx* c = detail::context(detail::params_of(param, param.lApprox));
    yg_key* key = detail::device_key_group(c, bsk.bskDft, bsk.group, &ksk, param.k, N);
    std::vector<int32_t> in(static_cast<size_t>(n) + 1), res(static_cast<size_t>(n) + 1);
    for (int i = 0; i < n; i++) in[i] = static_cast<int32_t>(input.a[i]);
    in[n] = static_cast<int32_t>(input.b);
    std::vector<int64_t> lut(N);
    for (int j = 0; j < N; j++) lut[j] = static_cast<int64_t>(v.coeffs[j]);
    detail::check(yg_pbs_host(c, key, in.data(), res.data(), 1, lut.data(), nullptr));
    if (out.a.size() != static_cast<size_t>(n)) out = Tlwe{n};
    for (int i = 0; i < n; i++) out.a[i] = static_cast<LweTorus>(res[i]);
    out.b = static_cast<LweTorus>(res[n]);
}

// blindRotateLazyPipeAltNttSweep: the same rotation with another split of the reference's
// CPU pipeline (moveNtt, unitsA), which does not change its result.
inline void blindRotateLazyPipeAltNttSweep(Trlwe& accum, const BootstrappingKeyMPLazyPipeAlt& bsk,
                                           const ScaledTlwe& input, const TorusPolynomial& v,
                                           const std::vector<NttPolynomial>& gdVntt, int moveNtt, int unitsA,
                                           const YatfheParameters& param) {
    // the splits only shape the reference's CPU pipeline (every split gives the same result);
    // the reference sizes its buffers by them, so non-positive ones are refused here
    if (moveNtt < 1 || unitsA < 1)
        throw std::invalid_argument("blindRotateLazyPipeAltNttSweep: moveNtt and unitsA must be >= 1");
    yatfhe_gb300::blindRotateLazyPipeAltNtt(accum, bsk, input, v, gdVntt, param);
}

// blindRotateLazyPipeAltInitNtt: the key read from fileName into bsk (the reference reads it
// while it rotates), then the same rotation on the GPU.  Like the reference, every call reads
// the file; every call also uploads and converts the key again (about 45 MB at the default
// T32 set), so a caller rotating many inputs under one file should read it once and call
// blindRotateLazyPipeAltNtt.
inline void blindRotateLazyPipeAltInitNtt(Trlwe& accum, BootstrappingKeyMPLazyPipeAlt& bsk, const ScaledTlwe& input,
                                          const TorusPolynomial& v, const std::string& fileName,
                                          const std::vector<NttPolynomial>& gdVntt, const YatfheParameters& param) {
    deserializeBskLazyPipeAlt(bsk, fileName, param.n);
    {
        auto& r = detail::reg();
        std::lock_guard<std::mutex> g(r.mu);
        auto it = r.keys.find(&bsk);
        if (it != r.keys.end()) {  // a key cached for this object before it was read again
            yg_key_destroy(it->second.key);
            r.keys.erase(it);
        }
    }
    yatfhe_gb300::blindRotateLazyPipeAltNtt(accum, bsk, input, v, gdVntt, param);
}

// blindRotateLazyPipeAltNoFirstNtt: the first key index through the ordinary chain instead of
// the first-component shortcut.  Both give the same accumulator bit for bit (the shortcut is
// that chain's first external product, the same polynomial mod q before the one rounding;
// tests/test_lazy_oracle.py checks it on the reference itself), so the GPU lazy rotation
// serves it.
inline void blindRotateLazyPipeAltNoFirstNtt(Trlwe& accum, const BootstrappingKeyMPLazyPipeAlt& bsk,
                                             const ScaledTlwe& input, const TorusPolynomial& v,
                                             const YatfheParameters& param) {
    yatfhe_gb300::blindRotateLazyPipeAltNtt(accum, bsk, input, v, {}, param);
}

inline void blindRotateJP22Ntt(Trlwe& accum, const BootstrappingKeyMP& bsk, const ScaledTlwe& input,
                               const YatfheParameters& param) {
    yatfhe_gb300::blindRotateMP21Ntt(accum, bsk.bskDft, input, param);
}

namespace detail {

// BootstrappingKeyCRT::bskCRT (yatfhe/include/yatfhe/bootstrapping.h:351-361) -> the residue rows
// [n][d][dh][k+1][k+1][N] (int8) the device key is made from: the reference's inverse NTT24 with
// the reduction mod q_d (NttNative24::applyIntt) returns the rows the NTT24 forms were made of.
inline std::vector<int8_t> flatten_crt(const std::vector<std::vector<TrgswDft24>>& bskCRT, const YatfheParameters& p) {
    const int N = p.N, k = p.k;
    std::vector<int8_t> out;
    out.reserve(bskCRT.size() * p.d * p.dh * (k + 1) * (k + 1) * (size_t)N);
    Int8Polynomial poly{N};
    for (const auto& perPrime : bskCRT) {
        if ((int)perPrime.size() != p.d) throw std::invalid_argument("bskCRT: one TrgswDft24 per prime");
        for (int d = 0; d < p.d; d++) {
            const TrgswDft24& t = perPrime[d];
            if (t.l < p.dh) throw std::invalid_argument("bskCRT: fewer levels than dh");
            for (int l = 0; l < p.dh; l++)
                for (int r = 0; r <= k; r++) {
                    const auto& row = t.trlweDftSamples[l][r];
                    for (int c = 0; c <= k; c++) {
                        NttNative24::applyIntt(poly, c < k ? row.a[c] : row.b, p.qd[d]);
                        out.insert(out.end(), poly.coeffs.begin(), poly.coeffs.end());
                    }
                }
        }
    }
    return out;
}

inline uint64_t fingerprint(const std::vector<std::vector<TrgswDft24>>& bskCRT) {
    uint64_t h = mix(0x43525400ULL, bskCRT.size());
    for (size_t i : probes(bskCRT))
        for (const auto& t : bskCRT[i]) {
            h = mix(h, t.trlweDftSamples.size());
            for (const auto& lvl : t.trlweDftSamples)
                for (const auto& row : lvl) {
                    h = mix_poly(h, row.b);
                    for (const auto& a : row.a) h = mix_poly(h, a);
                }
        }
    return h;
}

}  // namespace detail

// blindRotateApproxCRTNtt: accum (d residue samples, as decompTrlweMcrt leaves them) rotated in
// place.  The samples go to torus values mod Q_CRT (trlweMcrtToCrt + recompTrlweCrt on a copy)
// and come back by decompTrlweMcrt; on centred residues the two conversions invert each other,
// and the GPU entry point applies the same pair around the rotation.
inline void blindRotateApproxCRTNtt(std::vector<Trlwe8>& accum, const std::vector<std::vector<TrgswDft24>>& bskCRT,
                                    const ScaledTlwe& input, const YatfheParameters& param) {
    if (param.k != 1) throw std::invalid_argument("blindRotateApproxCRTNtt: k = 1 only");
    if ((int)accum.size() != param.d) throw std::invalid_argument("blindRotateApproxCRTNtt: one Trlwe8 per prime");
    if ((int)bskCRT.size() < input.n || input.n != param.n)
        throw std::invalid_argument("blindRotateApproxCRTNtt: key and input sizes differ");
    const int N = param.N;
    yg_crt_key* key = nullptr;
    {
        auto& r = detail::reg();
        std::lock_guard<std::mutex> g(r.mu);
        const uint64_t fp = detail::fingerprint(bskCRT);
        auto it = r.crt_keys.find(&bskCRT);
        if (it != r.crt_keys.end() && it->second.fp != fp) {
            yg_crt_key_destroy(it->second.key);
            r.crt_keys.erase(it);
            it = r.crt_keys.end();
        }
        if (it == r.crt_keys.end()) {
            const std::vector<int8_t> rows = detail::flatten_crt(bskCRT, param);
            yg_crt_key* k = nullptr;
            detail::check(yg_crt_key_upload(0, param.n, N, rows.data(), &k));
            it = r.crt_keys.emplace(&bskCRT, detail::CachedCrtKey{k, fp}).first;
        }
        key = it->second.key;
    }
    std::vector<Trlwe8> tmp = accum;
    trlweMcrtToCrt(tmp, param);
    Trlwe t{param.k, N};
    recompTrlweCrt(t, tmp, param);
    std::vector<int32_t> acc(2 * (size_t)N), rot(input.a.begin(), input.a.begin() + param.n);
    for (int j = 0; j < N; j++) {
        acc[j] = static_cast<int32_t>(t.a[0].coeffs[j]);
        acc[N + j] = static_cast<int32_t>(t.b.coeffs[j]);
    }
    detail::DeviceBuf<int32_t> d_acc(acc.size()), d_rot(rot.size()), d_out(acc.size());
    detail::cuda(cudaMemcpy(d_acc.p, acc.data(), acc.size() * 4, cudaMemcpyHostToDevice));
    detail::cuda(cudaMemcpy(d_rot.p, rot.data(), rot.size() * 4, cudaMemcpyHostToDevice));
    detail::check(yg_crt_blind_rotate(key, d_acc.p, d_rot.p, 1, d_out.p, nullptr));
    detail::cuda(cudaMemcpy(acc.data(), d_out.p, acc.size() * 4, cudaMemcpyDeviceToHost));
    for (int j = 0; j < N; j++) {
        t.a[0].coeffs[j] = static_cast<Torus>(acc[j]);
        t.b.coeffs[j] = static_cast<Torus>(acc[N + j]);
    }
    decompTrlweMcrt(accum, t, param);
}

inline void switchKeyForTlwe(Tlwe& output, const TlweKeySwitchingKey& ksk, const Tlwe& input,
                             const YatfheParameters& param) {
    // the key-switching key alone: attach it to a context-level key slot keyed by its address
    auto& r = detail::reg();
    std::lock_guard<std::mutex> g(r.mu);
    yg_ctx* c = detail::context(detail::params_of(param, param.lApprox));
    auto it = r.keys.find(&ksk);
    if (it == r.keys.end()) {
        yg_key* key = nullptr;
        detail::check(yg_key_create_ksk_only(c, &key));
        it = r.keys.emplace(&ksk, detail::CachedKey{key, 0, nullptr, 0}).first;
    }
    detail::attach_ksk(it->second, ksk);
    yg_key* key = it->second.key;
    const int kN = param.k * param.N, n = param.n;
    std::vector<int32_t> big(kN + 1), res(n + 1);
    for (int j = 0; j < kN; j++) big[j] = static_cast<int32_t>(input.a[j]);
    big[kN] = static_cast<int32_t>(input.b);
    detail::DeviceBuf<int32_t> d_big(big.size()), d_out(res.size());
    detail::cuda(cudaMemcpy(d_big.p, big.data(), big.size() * 4, cudaMemcpyHostToDevice));
    detail::check(yg_keyswitch(c, key, d_big.p, d_out.p, 1, nullptr));
    detail::cuda(cudaMemcpy(res.data(), d_out.p, res.size() * 4, cudaMemcpyDeviceToHost));
    for (int j = 0; j < n; j++) output.a[j] = static_cast<LweTorus>(res[j]);
    output.b = static_cast<LweTorus>(res[n]);
}

}  // namespace yatfhe_gb300

#endif  // YATFHE_GB300_REFERENCE_HPP
