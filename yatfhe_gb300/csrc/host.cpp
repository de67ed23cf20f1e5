// host.cpp -- C ABI of the GB300 bootstrap (include/yatfhe_gb300.h): contexts, key
// loading and conversion, launches.
//
// Key conversion.  The reference stores bootstrapping keys in the NTT domain of its
// 64-bit prime q (serializeBskMP, yatfhe/src/ya_serializer.cpp:276-285; the words come
// from HEXL's forward transform, yatfhe/include/yatfhe/ntt_hexl.h:34-44).  Every CMux
// only ever uses them through centred(INTT(sum NTT(d) . K) mod q) (ntt_hexl.cpp:153-175),
// so the loader takes each key polynomial back to coefficients once (inverse negacyclic
// transform mod q with the minimal primitive 2N-th root, bit-reversed slot order: the
// convention HEXL documents), centres them and reduces them into the three RNS channels
// (key_intt_kernel, on the GPU, with the tables QTables builds here), and keyconv_kernel
// applies the GPU's own per-channel NTT.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/yatfhe_gb300.h"
#include "internal.hpp"
#include "pbs_kernels.cuh"

std::string& yg::last_error_slot() {
    thread_local std::string msg;
    return msg;
}

namespace {

using u64 = uint64_t;
using u128 = unsigned __int128;
using yg::ck;
using yg::CudaError;
using yg::DeviceGuard;
using yg::guarded;
using yg::set_err;

u64 mulmod(u64 a, u64 b, u64 m) { return (u64)((u128)a * b % m); }
u64 powmod(u64 b, u64 e, u64 m) {
    u64 r = 1 % m;
    b %= m;
    while (e) {
        if (e & 1) r = mulmod(r, b, m);
        b = mulmod(b, b, m);
        e >>= 1;
    }
    return r;
}
u64 invmod(u64 a, u64 p) { return powmod(a, p - 2, p); }
uint32_t brv(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int i = 0; i < bits; i++) r = (r << 1) | ((x >> i) & 1);
    return r;
}

// Smallest primitive 2N-th root of unity mod a prime m == 1 (mod 2N).
u64 minimal_root(u64 N, u64 m) {
    const u64 twoN = 2 * N;
    u64 psi0 = 0;
    for (u64 x = 2; x < m && !psi0; x++) {
        const u64 c = powmod(x, (m - 1) / twoN, m);
        if (powmod(c, N, m) == m - 1) psi0 = c;
    }
    if (!psi0) throw std::invalid_argument("no primitive 2N-th root of unity");
    u64 best = psi0, cur = psi0;
    const u64 sq = mulmod(psi0, psi0, m);
    for (u64 k = 1; k < N; k++) {
        cur = mulmod(cur, sq, m);
        best = std::min(best, cur);
    }
    return best;
}

uint32_t shoup32(uint32_t w, uint32_t p) { return (uint32_t)(((u64)w << 32) / p); }

// Reorders one twiddle table (N entries, index order psi^brv(k)) into the layout the team
// NTT reads (ntt.cuh): the per-thread entries of each slot-layout stage, 2^(9-sp) + gid K + k
// with K = 2^(4-sp), move to 2^(9-sp) + k 32 + gid; at N = 2048 the index-bit-0 stage's
// 1024 + gid 32 + r moves to 1024 + r 32 + gid.  Entries 0..31 stay.
void thread_minor_layout(uint2* t, int N) {
    std::vector<uint2> src(t, t + N);
    auto region = [&](int base, int K) {
        for (int gid = 0; gid < 32; gid++)
            for (int k = 0; k < K; k++) t[base + k * 32 + gid] = src[base + gid * K + k];
    };
    for (int sp = 0; sp <= 4; sp++) region(1 << (9 - sp), 1 << (4 - sp));
    if (N == 2048) region(1024, 32);
}

}  // namespace

namespace yg {

// Tables of the negacyclic transforms mod q the key kernels run: the inverse
// (Gentleman-Sande, psi^-brv(k) twiddles, bit-reversed NTT slots in, natural-order
// coefficients out, times N^-1) and the forward one (Cooley-Tukey, psi^brv(k)), with Shoup
// companions, psi the minimal primitive 2N-th root of unity mod q.
struct QTables {
    int N = 0, logN = 0;
    u64 q = 0;
    std::vector<u64> w, wp;    // inverse
    std::vector<u64> wf, wfp;  // forward
    u64 ninv = 0, ninvp = 0;

    QTables(int N_, u64 q_) : N(N_), q(q_) {
        while ((1 << logN) < N) logN++;
        const u64 psi = minimal_root(N, q), psi_inv = invmod(psi, q);
        w.resize(N);
        wp.resize(N);
        wf.resize(N);
        wfp.resize(N);
        for (int k = 0; k < N; k++) {
            w[k] = powmod(psi_inv, brv(k, logN), q);
            wp[k] = (u64)(((u128)w[k] << 64) / q);
            wf[k] = powmod(psi, brv(k, logN), q);
            wfp[k] = (u64)(((u128)wf[k] << 64) / q);
        }
        ninv = invmod(N, q);
        ninvp = (u64)(((u128)ninv << 64) / q);
    }
};

}  // namespace yg

namespace {

using yg::QTables;

void validate(const yg_params& p) {
    if (p.torus_bits != 32 && p.torus_bits != 56) throw std::invalid_argument("torus_bits must be 32 or 56");
    if (p.N != 1024 && p.N != 2048) throw std::invalid_argument("N must be 1024 or 2048");
    if (p.k != 1) throw std::invalid_argument("only k = 1 is supported");
    if (p.n < 1 || p.n > 4096) throw std::invalid_argument("n must be in [1, 4096]");
    if (p.l_approx < 1 || p.radix_bits < 1 || p.l_approx * p.radix_bits > p.torus_bits)
        throw std::invalid_argument("decomposeRow: l * radixBits exceeds the torus width");
    if (p.radix_bits > 15) throw std::invalid_argument("radix_bits must be <= 15 (int16 digits)");
    // the channel-row layout at T = 32 sums 2 l products of transform outputs (< 46p) and
    // key words (< p) exactly in 64 bits: below 2^64 for l <= 15
    if (p.l_approx > 15) throw std::invalid_argument("l must be <= 15");
    if (p.ks_level < 1 || p.ks_level > 16 || p.ks_radix_bits < 1 || p.ks_level * p.ks_radix_bits > 32 ||
        p.ks_radix_bits > 7)
        throw std::invalid_argument("key-switching decomposition must fit 32 bits, t <= 16, radix <= 7");
    // exactness of the three-prime RNS: |X| <= (B/2)(q/2)(k+1) l N must stay below M/2
    const double q = p.torus_bits == 32 ? 562941363486721.0 : 1945555039024054273.0;
    const double bound = std::ldexp(1.0, p.radix_bits - 1) * (q / 2) * (p.k + 1) * p.l_approx * p.N;
    const uint32_t* P = yg::kPrimeSet[yg::prime_set_for(p.torus_bits)];
    const double M = (double)P[0] * P[1] * P[2];
    if (bound >= M / 4) throw std::invalid_argument("parameters exceed the exact range of the RNS");
}

// Twiddle tables of the team NTT (ntt.cuh), per channel [forward N | inverse 2N]:
//   forward: psi^brv(k), thread-minor (thread_minor_layout); its first 32 entries also go to
//            the constant bank;
//   inverse, Cooley-Tukey form (prime set 1, N = 1024): entries 32 (2^sp - 1) + m 32 + tt =
//            psi^-((N / 2^(5+sp)) (m 32 + tt)) for the stages on index bits 5 + sp, then
//            992 + j = psi^-j (the twist); the constant bank gets psi^-((N / 2^sp) m) at
//            2^sp + m for the stages on slot bits sp = 1..4 (entry 1: the twiddle 1 of bit 0);
//   inverse, Gentleman-Sande form (the other shapes): psi^-brv(k), thread-minor, first 32
//            entries to the constant bank.
// One prime's tables: tw [N forward | 2N inverse], heads [forward 32 | inverse 32].
void team_tables(uint32_t p, int N, int logN, bool ct_inverse, uint2* tw, uint2* heads) {
    const u64 psi = minimal_root(N, p);
    const u64 psi_inv = invmod(psi, p);
    uint2* fwd = tw;
    uint2* inv = fwd + N;
    auto pair = [p](u64 w) { return make_uint2((uint32_t)w, shoup32((uint32_t)w, p)); };
    for (int k = 0; k < N; k++) {
        const uint32_t e = brv(k, logN);
        fwd[k] = pair(powmod(psi, e, p));
        if (!ct_inverse) inv[k] = pair(powmod(psi_inv, e, p));
    }
    thread_minor_layout(fwd, N);
    for (int k = 0; k < 32; k++) heads[k] = fwd[k];
    if (ct_inverse) {
        for (int sp = 0; sp <= 4; sp++) {
            const int h = 1 << sp;
            for (int m = 0; m < h; m++)
                for (int tt = 0; tt < 32; tt++)
                    inv[32 * (h - 1) + m * 32 + tt] = pair(powmod(psi_inv, (u64)(N / (32 * h)) * (m * 32 + tt), p));
        }
        for (int j = 0; j < N; j++) inv[992 + j] = pair(powmod(psi_inv, j, p));
        uint2* hd = heads + 32;
        hd[0] = hd[1] = pair(1);
        for (int sp = 1; sp <= 4; sp++)
            for (int m = 0; m < (1 << sp); m++) hd[(1 << sp) + m] = pair(powmod(psi_inv, (u64)(N >> sp) * m, p));
    } else {
        thread_minor_layout(inv, N);
        for (int k = 0; k < 32; k++) heads[32 + k] = inv[k];
    }
}

// Montgomery form with N^-1 folded in: N^-1 2^32 mod p
uint32_t conv_scale_for(uint32_t p, int N) { return (uint32_t)mulmod(invmod(N, p), ((u64)1 << 32) % p, p); }

uint32_t neg_pinv32(uint32_t p) {
    uint32_t pinv = 1;  // p^-1 mod 2^32 by Newton iteration
    for (int it = 0; it < 5; it++) pinv *= 2 - p * pinv;
    return 0u - pinv;
}

void ctx_init_tables(yg_ctx* c) {
    const int N = c->p.N;
    const size_t per = (size_t)3 * N;  // words of one channel's tables
    const bool ct_inverse = c->ps == 1 && N == 1024;
    std::vector<uint2> tw((size_t)yg::kChannels * per);
    std::vector<uint2> heads((size_t)yg::kChannels * 2 * 32);
    for (int ci = 0; ci < yg::kChannels; ci++) {
        const uint32_t p = yg::kPrimeSet[c->ps][ci];
        team_tables(p, N, c->logN, ct_inverse, &tw[ci * per], &heads[(size_t)ci * 2 * 32]);
        const uint32_t sc = conv_scale_for(p, N);
        c->conv_scale[ci] = sc;
        c->conv_scale_s[ci] = shoup32(sc, p);
    }
    ck(cudaMalloc(&c->d_tw, tw.size() * sizeof(uint2)), "cudaMalloc twiddles");
    ck(cudaMemcpy(c->d_tw, tw.data(), tw.size() * sizeof(uint2), cudaMemcpyHostToDevice), "upload twiddles");
    if (ct_inverse) {
        // the 16-residue inverse of the channel-cluster layout: psi^-e in natural order
        std::vector<uint2> t16((size_t)yg::kChannels * N);
        for (int ci = 0; ci < yg::kChannels; ci++) {
            const uint32_t p = yg::kPrimeSet[c->ps][ci];
            const u64 psi_inv = invmod(minimal_root(N, p), p);
            for (int k = 0; k < N; k++) {
                const uint32_t wi = (uint32_t)powmod(psi_inv, k, p);
                t16[(size_t)ci * N + k] = make_uint2(wi, shoup32(wi, p));
            }
        }
        ck(cudaMalloc(&c->d_tw16, t16.size() * sizeof(uint2)), "cudaMalloc twiddles");
        ck(cudaMemcpy(c->d_tw16, t16.data(), t16.size() * sizeof(uint2), cudaMemcpyHostToDevice), "upload twiddles");
    }
    if (yg::set_twiddle_heads(c->logN, c->ps, heads.data()) != 0) ck(cudaGetLastError(), "upload twiddle heads");
    for (int ci = 0; ci < yg::kChannels; ci++) {
        const uint32_t p = yg::kPrimeSet[c->ps][ci];
        c->ch[ci] = yg::Chan{p, 2 * p, neg_pinv32(p), 0, c->d_tw + ci * per, c->d_tw + ci * per + N};
    }
    const u64 p0 = yg::kPrimeSet[c->ps][0], p1 = yg::kPrimeSet[c->ps][1], p2 = yg::kPrimeSet[c->ps][2];
    yg::Crt& k = c->crt;
    k.p0 = (uint32_t)p0;
    k.p1 = (uint32_t)p1;
    k.p2 = (uint32_t)p2;
    k.inv_p0_m1 = (uint32_t)invmod(p0 % p1, p1);
    k.inv_p0_m1_s = shoup32(k.inv_p0_m1, (uint32_t)p1);
    k.p0_m2 = (uint32_t)(p0 % p2);
    k.p0_m2_s = shoup32(k.p0_m2, (uint32_t)p2);
    k.inv_p01_m2 = (uint32_t)invmod(mulmod(p0, p1, p2), p2);
    k.inv_p01_m2_s = shoup32(k.inv_p01_m2, (uint32_t)p2);
    k.half_p2 = (uint32_t)((p2 - 1) / 2);
    k.p01 = p0 * p1;
    k.q = c->q;
    k.half_q = (c->q - 1) / 2;
    k.a2 = (int64_t)((((u128)k.p01 << 32) + c->q / 2) / c->q);
    k.a1 = (uint32_t)((((u128)p0 << 32) + c->q / 2) / c->q);
}

// NTT-domain key words -> device key.  Layout in: [n][L][k+1][k+1][N] u64.
// Device scratch freed on every exit path.
struct DeviceScratch {
    std::vector<void*> ptrs;
    template <typename T>
    T* alloc(size_t count, const char* what) {
        void* p = nullptr;
        ck(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), what);
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~DeviceScratch() {
        for (void* p : ptrs) cudaFree(p);
    }
};

// The mod-q transform tables on the device, for the key kernels.
struct DeviceQTables {
    u64 *w, *wp, *wf, *wfp;
    DeviceQTables(DeviceScratch& scratch, const QTables& qt) {
        const int N = qt.N;
        w = scratch.alloc<u64>(4 * (size_t)N, "cudaMalloc mod-q twiddles");
        wp = w + N;
        wf = wp + N;
        wfp = wf + N;
        const std::vector<u64>* src[4] = {&qt.w, &qt.wp, &qt.wf, &qt.wfp};
        for (int t = 0; t < 4; t++)
            ck(cudaMemcpy(w + (size_t)t * N, src[t]->data(), N * sizeof(u64), cudaMemcpyHostToDevice),
               "upload mod-q twiddles");
    }
};

// NTT-domain key words already on the device ([n][L][k+1][k+1][N]) -> the device key.
void convert_bsk_words(yg_ctx* c, yg_key* key, const u64* d_words, DeviceScratch& scratch, const DeviceQTables& tw) {
    const int n = c->p.n, N = c->p.N, L = c->p.l_approx;
    const size_t polys = (size_t)n * L * 2 * 2;
    const QTables& qi = *c->qtab;
    const size_t key_words = yg::key_words(n, L, N);
    key->bsk_bytes = key_words * sizeof(uint32_t);
    ck(cudaMalloc(&key->d_bsk, key->bsk_bytes), "cudaMalloc bsk");
    uint32_t* d_res = scratch.alloc<uint32_t>(polys * yg::kChannels * N, "cudaMalloc key residues");
    int* d_bad = scratch.alloc<int>(1, "cudaMalloc flag");
    const u64* d_w = tw.w;
    const u64* d_wp = tw.wp;
    ck(cudaMemset(d_bad, 0, sizeof(int)), "clear flag");
    yg::KeyInttArgs ia{};
    ia.words = d_words;
    ia.residues = d_res;
    ia.w = d_w;
    ia.wp = d_wp;
    ia.q = c->q;
    ia.ninv = qi.ninv;
    ia.ninvp = qi.ninvp;
    for (int ci = 0; ci < yg::kChannels; ci++) ia.p[ci] = yg::kPrimeSet[c->ps][ci];
    ia.N = N;
    ia.polys = (int)polys;
    ia.bad = d_bad;
    yg::check_launch(yg::launch_key_intt(ia, nullptr), "key inverse-transform launch");
    int bad = 0;
    ck(cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost), "key inverse transform");
    if (bad) throw std::invalid_argument("key word not reduced mod q");
    yg::KeyConvArgs a{};
    a.residues = d_res;
    a.key = key->d_bsk;
    a.polys = (int)polys;
    for (int ci = 0; ci < yg::kChannels; ci++) {
        a.ch[ci] = c->ch[ci];
        a.scale[ci] = c->conv_scale[ci];
        a.scale_s[ci] = c->conv_scale_s[ci];
    }
    yg::check_launch(yg::launch_keyconv(c->logN, c->ps, a, nullptr), "keyconv launch");
    ck(cudaDeviceSynchronize(), "keyconv");
}

// NTT-domain key words mod q -> the device key: the words go to the GPU as they are, the
// inverse transform mod q and the split into channel residues run there (key_intt_kernel),
// then keyconv_kernel applies each channel's forward NTT into the slot layout.
void upload_bsk(yg_ctx* c, yg_key* key, const u64* words) {
    const size_t polys = (size_t)c->p.n * c->p.l_approx * 2 * 2;
    DeviceScratch scratch;
    DeviceQTables tw(scratch, *c->qtab);
    u64* d_words = scratch.alloc<u64>(polys * c->p.N, "cudaMalloc key words");
    ck(cudaMemcpy(d_words, words, polys * c->p.N * sizeof(u64), cudaMemcpyHostToDevice), "upload key words");
    convert_bsk_words(c, key, d_words, scratch, tw);
}

// WWL+24 half key -> the device key.  The key's cPrime rows ([n][L][2][N]) and s2 key
// ([l][2][N]) go to the GPU, wwl24_expand_kernel derives the GINX rows blindRotateWWL24Ntt
// would build at every step (switchTrlweToSecretEmbeddingNtt, yatfhe/src/trgsw.cpp:861-905)
// once for the whole key, and the result is converted like any NTT-domain key.
void upload_wwl24(yg_ctx* c, yg_key* key, const u64* cprime, const u64* s2, int Ls) {
    const int n = c->p.n, N = c->p.N, L = c->p.l_approx;
    if (Ls < 1 || Ls > yg::kWwlMaxLevels || Ls * c->p.radix_bits > c->p.torus_bits)
        throw std::invalid_argument("WWL+24 s2 key: 1 <= levels <= 8 and levels * radix_bits <= torus_bits");
    const u64 q = c->q;
    const size_t s2_words = (size_t)Ls * 2 * N, cp_words = (size_t)n * L * 2 * N;
    std::vector<u64> s2p(s2_words);
    for (size_t j = 0; j < s2_words; j++) {
        if (s2[j] >= q) throw std::invalid_argument("WWL+24 s2 key word not reduced mod q");
        s2p[j] = (u64)(((u128)s2[j] << 64) / q);
    }
    DeviceScratch scratch;
    DeviceQTables tw(scratch, *c->qtab);
    u64* d_cp = scratch.alloc<u64>(cp_words, "cudaMalloc WWL+24 key");
    u64* d_s2 = scratch.alloc<u64>(2 * s2_words, "cudaMalloc WWL+24 s2 key");
    u64* d_out = scratch.alloc<u64>(2 * cp_words, "cudaMalloc expanded key");
    int* d_bad = scratch.alloc<int>(1, "cudaMalloc flag");
    ck(cudaMemcpy(d_cp, cprime, cp_words * sizeof(u64), cudaMemcpyHostToDevice), "upload WWL+24 key");
    ck(cudaMemcpy(d_s2, s2, s2_words * sizeof(u64), cudaMemcpyHostToDevice), "upload WWL+24 s2 key");
    ck(cudaMemcpy(d_s2 + s2_words, s2p.data(), s2_words * sizeof(u64), cudaMemcpyHostToDevice), "upload s2 key");
    ck(cudaMemset(d_bad, 0, sizeof(int)), "clear flag");
    yg::WwlExpandArgs a{};
    a.cprime = d_cp;
    a.s2 = d_s2;
    a.s2p = d_s2 + s2_words;
    a.out = d_out;
    a.wi = tw.w;
    a.wip = tw.wp;
    a.wf = tw.wf;
    a.wfp = tw.wfp;
    a.q = q;
    a.ninv = c->qtab->ninv;
    a.ninvp = c->qtab->ninvp;
    a.n = n;
    a.N = N;
    a.L = L;
    a.Ls = Ls;
    a.radix_bits = c->p.radix_bits;
    a.torus_bits = c->p.torus_bits;
    a.bad = d_bad;
    yg::check_launch(yg::launch_wwl24_expand(a, nullptr), "WWL+24 key expansion launch");
    int bad = 0;
    ck(cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost), "WWL+24 key expansion");
    if (bad) throw std::invalid_argument("WWL+24 key word not reduced mod q");
    convert_bsk_words(c, key, d_out, scratch, tw);
}

int64_t sext_host(int64_t x, int bits) { return (int64_t)((uint64_t)x << (64 - bits)) >> (64 - bits); }

// Lazy key -> the device: the half rows ([n][L][2][N] torus values) in the torus word size,
// and the mod-q transform tables with the s2 key ([Ls][2][N] NTT-domain words) and their
// Shoup companions.  The blind rotation rebuilds each step's rows from these
// (lazy_blind_rotate_kernel); no other conversion runs at upload.
void upload_lazy(yg_ctx* c, yg_key* key, const int64_t* cprime, const u64* s2, int Ls) {
    const int n = c->p.n, N = c->p.N, L = c->p.l_approx, T = c->p.torus_bits, rb = c->p.radix_bits;
    if (n < 2) throw std::invalid_argument("lazy key: the blind rotation needs n >= 2");
    if (L > yg::kLazyMaxLevels) throw std::invalid_argument("lazy key: l_approx <= 8");
    if (rb > 15) throw std::invalid_argument("lazy key: radix_bits <= 15");
    if (Ls < 1 || Ls > yg::kLazyMaxLevels || Ls * rb > T)
        throw std::invalid_argument("lazy s2 key: 1 <= levels <= 8 and levels * radix_bits <= torus_bits");
    const u64 q = c->q;
    const QTables& qt = *c->qtab;
    const size_t s2_words = (size_t)Ls * 2 * N, cp_words = (size_t)n * L * 2 * N;
    std::vector<u64> tab(4 * (size_t)N + 2 * s2_words);
    std::copy(qt.w.begin(), qt.w.end(), tab.begin());
    std::copy(qt.wp.begin(), qt.wp.end(), tab.begin() + N);
    std::copy(qt.wf.begin(), qt.wf.end(), tab.begin() + 2 * (size_t)N);
    std::copy(qt.wfp.begin(), qt.wfp.end(), tab.begin() + 3 * (size_t)N);
    u64* t2 = tab.data() + 4 * (size_t)N;
    for (size_t j = 0; j < s2_words; j++) {
        if (s2[j] >= q) throw std::invalid_argument("lazy s2 key word not reduced mod q");
        t2[j] = s2[j];
        t2[s2_words + j] = (u64)(((u128)s2[j] << 64) / q);
    }
    const size_t wb = T == 32 ? 4 : 8;
    std::vector<unsigned char> words(cp_words * wb);
    for (size_t j = 0; j < cp_words; j++) {
        const int64_t v = cprime[j];
        if (sext_host(v, T) != v) throw std::invalid_argument("lazy key word is not a sign-extended torus value");
        if (T == 32) {
            const int32_t w = (int32_t)v;
            std::memcpy(words.data() + j * 4, &w, 4);
        } else {
            std::memcpy(words.data() + j * 8, &v, 8);
        }
    }
    ck(cudaMalloc(&key->d_lazy_tab, tab.size() * sizeof(u64)), "cudaMalloc lazy tables");
    ck(cudaMalloc(&key->d_lazy_cprime, words.size()), "cudaMalloc lazy key");
    ck(cudaMemcpy(key->d_lazy_tab, tab.data(), tab.size() * sizeof(u64), cudaMemcpyHostToDevice), "upload lazy tables");
    ck(cudaMemcpy(key->d_lazy_cprime, words.data(), words.size(), cudaMemcpyHostToDevice), "upload lazy key");
    key->lazy_ls = Ls;
    key->bsk_bytes = tab.size() * sizeof(u64) + words.size();
}

// Group-g key (TrgswDft words [keys][key_levels][2][2][N]) -> the device: the levels the
// external product uses (l_approx of them), the mod-q transform tables, psi^j 2^64 mod q for
// j < 2N and the exponent e_s of every transform slot (slot s of NTT(X^r) is psi^(r e_s)),
// found by transforming X on the host with the kernels' forward transform.
void upload_group(yg_ctx* c, yg_key* key, const u64* words, int group, int key_levels) {
    const int n = c->p.n, N = c->p.N, L = c->p.l_approx, rb = c->p.radix_bits, T = c->p.torus_bits;
    if (group < 1 || group > 3 || n % group) throw std::invalid_argument("group key: group 1, 2 or 3, dividing n");
    if (key_levels < L || key_levels > yg::kGroupMaxLevels || key_levels * rb > T)
        throw std::invalid_argument("group key: l_approx <= key levels <= 8 and key levels * radix_bits <= torus_bits");
    const u64 q = c->q;
    const QTables& qt = *c->qtab;
    const size_t keys = group == 1 ? (size_t)n : (size_t)(n / group) << group;
    const size_t used = (size_t)L * 4 * N, full = (size_t)key_levels * 4 * N;
    std::vector<u64> w(keys * used);
    for (size_t j = 0; j < keys; j++)
        for (size_t x = 0; x < used; x++) {
            const u64 v = words[j * full + x];
            if (v >= q) throw std::invalid_argument("group key word not reduced mod q");
            w[j * used + x] = v;
        }
    // slot exponents: the forward transform of X, then each slot's power of psi
    std::vector<u64> x(N, 0);
    x[1] = 1;
    for (int m = 1, t = N / 2; m < N; m <<= 1, t >>= 1)
        for (int b = 0; b < N / 2; b++) {
            const int i = b / t, j = b - i * t, xi = 2 * i * t + j, yi = xi + t;
            const u64 u = x[xi], v = mulmod(x[yi], qt.wf[m + i], q);
            x[xi] = (u + v) % q;
            x[yi] = (u + q - v) % q;
        }
    const u64 psi = minimal_root(N, q);
    std::map<u64, int> expo;
    std::vector<u64> tab(7 * (size_t)N);
    u64 pw = 1;
    const u64 r64 = (u64)(((u128)1 << 64) % q);
    for (int j = 0; j < 2 * N; j++) {
        expo[pw] = j;
        tab[4 * (size_t)N + j] = mulmod(pw, r64, q);
        pw = mulmod(pw, psi, q);
    }
    for (int s = 0; s < N; s++) {
        auto it = expo.find(x[s]);
        if (it == expo.end() || !(it->second & 1)) throw std::runtime_error("slot exponent not found");
        tab[6 * (size_t)N + s] = (u64)it->second;
    }
    std::copy(qt.w.begin(), qt.w.end(), tab.begin());
    std::copy(qt.wp.begin(), qt.wp.end(), tab.begin() + N);
    std::copy(qt.wf.begin(), qt.wf.end(), tab.begin() + 2 * (size_t)N);
    std::copy(qt.wfp.begin(), qt.wfp.end(), tab.begin() + 3 * (size_t)N);
    ck(cudaMalloc(&key->d_group_tab, tab.size() * sizeof(u64)), "cudaMalloc group tables");
    ck(cudaMalloc(&key->d_group, w.size() * sizeof(u64)), "cudaMalloc group key");
    ck(cudaMemcpy(key->d_group_tab, tab.data(), tab.size() * sizeof(u64), cudaMemcpyHostToDevice), "upload group tables");
    ck(cudaMemcpy(key->d_group, w.data(), w.size() * sizeof(u64), cudaMemcpyHostToDevice), "upload group key");
    key->group = group;
    key->group_levels = key_levels;
    key->bsk_bytes = (tab.size() + w.size()) * sizeof(u64);
}

// Key generation arithmetic on the GPU from caller-drawn samples (see yg_keygen_from_samples):
// the NTT of the RLWE secret mod q (host, exact), the BSK samples (keygen_bsk_kernel), the
// usual conversion of the NTT-domain words, and the KSK samples (keygen_ksk_kernel).
// Device buffers of one key generation's samples (the layouts of yg_keygen_from_samples).
struct KeygenSamples {
    int32_t *lwe_s, *rlwe_s, *noise, *kmask, *knoise;
    u64* mask;
    size_t samples, ksk_samples;
};

KeygenSamples alloc_samples(const yg_ctx* c, DeviceScratch& scratch) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->p.l_approx, kN = k * N;
    KeygenSamples d{};
    d.samples = (size_t)n * L * (k + 1);
    d.ksk_samples = (size_t)kN * c->p.ks_level;
    d.lwe_s = scratch.alloc<int32_t>(n, "cudaMalloc keygen");
    d.rlwe_s = scratch.alloc<int32_t>(kN, "cudaMalloc keygen");
    d.noise = scratch.alloc<int32_t>(d.samples * N, "cudaMalloc keygen noise");
    d.mask = scratch.alloc<u64>(d.samples * k * N, "cudaMalloc keygen masks");
    d.kmask = scratch.alloc<int32_t>(d.ksk_samples * n, "cudaMalloc keygen KSK masks");
    d.knoise = scratch.alloc<int32_t>(d.ksk_samples, "cudaMalloc keygen KSK noise");
    return d;
}

// Domains of the GPU draws (sampling.cu): one ChaCha20 key per array of a draw.
enum : uint32_t { kDomLweS = 1, kDomRlweS, kDomBskNoise, kDomBskMask, kDomKskMask, kDomKskNoise, kDomEncrypt = 16 };

void draw(int32_t* out_i32, u64* out_u64, size_t count, uint64_t seed, uint32_t domain, int kind, int b, u64 q) {
    yg::DrawArgs a{};
    a.out_i32 = out_i32;
    a.out_u64 = out_u64;
    a.count = count;
    a.seed = seed;
    a.q = q;
    a.domain = domain;
    a.kind = kind;
    a.b = b;
    a.per_block = kind == yg::kDrawTUniform ? 8 : (kind == yg::kDrawModQ ? 4 : 16);
    yg::check_launch(yg::launch_draw(a, nullptr), "draw launch");
}

// Every sample of a key generation drawn on the GPU from `seed`, with the distributions of
// genTlweKey, genTrlweKey, encryptTrgswMPNtt (TUniform(rlwe_noise_b) noise, uniform masks mod
// q) and genTlweKeySwitchingKey (uniform 32-bit masks, TUniform(lwe_noise_b) noise).
void draw_keygen_samples(const yg_ctx* c, uint64_t seed, int lwe_noise_b, int rlwe_noise_b, const KeygenSamples& d) {
    if (lwe_noise_b < 0 || lwe_noise_b > 30 || rlwe_noise_b < 0 || rlwe_noise_b > 30)
        throw std::invalid_argument("noise widths: 0 <= lwe_noise_b, rlwe_noise_b <= 30");
    const int n = c->p.n, N = c->p.N, k = c->p.k;
    draw(d.lwe_s, nullptr, (size_t)n, seed, kDomLweS, yg::kDrawBit, 0, 0);
    draw(d.rlwe_s, nullptr, (size_t)k * N, seed, kDomRlweS, yg::kDrawBit, 0, 0);
    draw(d.noise, nullptr, d.samples * N, seed, kDomBskNoise, yg::kDrawTUniform, rlwe_noise_b, 0);
    draw(nullptr, d.mask, d.samples * k * N, seed, kDomBskMask, yg::kDrawModQ, 0, c->q);
    draw(d.kmask, nullptr, d.ksk_samples * n, seed, kDomKskMask, yg::kDrawU32, 0, 0);
    draw(d.knoise, nullptr, d.ksk_samples, seed, kDomKskNoise, yg::kDrawTUniform, lwe_noise_b, 0);
}

// The key from samples already on the device (the secret's transform is computed on the
// host from rlwe_s).
void keygen_on_device(yg_ctx* c, yg_key* key, const int32_t* rlwe_s, const KeygenSamples& d, u64* h_words,
                      int32_t* h_ksk, DeviceScratch& scratch) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, L = c->p.l_approx, t = c->p.ks_level, kN = k * N;
    const QTables& qt = *c->qtab;
    const u64 q = c->q;
    // NTT(s) mod q, the forward transform the kernels use (Cooley-Tukey, psi^brv twiddles)
    std::vector<u64> s_ntt((size_t)kN), s_ntt_p((size_t)kN);
    for (int r = 0; r < k; r++) {
        u64* a = s_ntt.data() + (size_t)r * N;
        for (int j = 0; j < N; j++) a[j] = (u64)rlwe_s[(size_t)r * N + j];
        for (int m = 1, span = N / 2; m < N; m <<= 1, span >>= 1)
            for (int g = 0; g < m; g++)
                for (int j = 2 * g * span; j < 2 * g * span + span; j++) {
                    const u64 u = a[j], v = mulmod(a[j + span], qt.wf[m + g], q);
                    a[j] = u + v >= q ? u + v - q : u + v;
                    a[j + span] = u >= v ? u - v : u + q - v;
                }
        for (int j = 0; j < N; j++) s_ntt_p[(size_t)r * N + j] = (u64)(((u128)a[j] << 64) / q);
    }
    const size_t words = d.samples * (k + 1) * N;
    DeviceQTables tw(scratch, qt);
    u64* d_s = scratch.alloc<u64>(2 * (size_t)kN, "cudaMalloc keygen secret");
    u64* d_words = scratch.alloc<u64>(words, "cudaMalloc keygen words");
    int* d_bad = scratch.alloc<int>(1, "cudaMalloc flag");
    ck(cudaMemcpy(d_s, s_ntt.data(), kN * sizeof(u64), cudaMemcpyHostToDevice), "upload keygen secret");
    ck(cudaMemcpy(d_s + kN, s_ntt_p.data(), kN * sizeof(u64), cudaMemcpyHostToDevice), "upload keygen secret");
    ck(cudaMemset(d_bad, 0, sizeof(int)), "clear flag");
    yg::KeygenBskArgs a{};
    a.lwe_s = d.lwe_s;
    a.noise = d.noise;
    a.mask = d.mask;
    a.s_ntt = d_s;
    a.s_ntt_p = d_s + kN;
    a.wf = tw.wf;
    a.wfp = tw.wfp;
    a.words = d_words;
    a.q = q;
    a.n = n;
    a.N = N;
    a.k = k;
    a.L = L;
    a.radix_bits = c->p.radix_bits;
    a.torus_bits = c->p.torus_bits;
    a.bad = d_bad;
    yg::check_launch(yg::launch_keygen_bsk(a, nullptr), "keygen launch");
    int bad = 0;
    ck(cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost), "keygen");
    if (bad) throw std::invalid_argument("BSK mask word not reduced mod q");
    if (h_words) ck(cudaMemcpy(h_words, d_words, words * sizeof(u64), cudaMemcpyDeviceToHost), "download BSK words");
    convert_bsk_words(c, key, d_words, scratch, tw);
    key->ksk_bytes = d.ksk_samples * (n + 1) * sizeof(int32_t);
    ck(cudaMalloc(&key->d_ksk, key->ksk_bytes), "cudaMalloc ksk");
    yg::KeygenKskArgs kk{d.lwe_s, d.rlwe_s, d.kmask, d.knoise, key->d_ksk, n, kN, t, c->p.ks_radix_bits};
    yg::check_launch(yg::launch_keygen_ksk(kk, nullptr), "keygen KSK launch");
    if (h_ksk) ck(cudaMemcpy(h_ksk, key->d_ksk, key->ksk_bytes, cudaMemcpyDeviceToHost), "download KSK");
    ck(cudaDeviceSynchronize(), "keygen");
}

void keygen_from_samples(yg_ctx* c, yg_key* key, const int32_t* lwe_s, const int32_t* rlwe_s, const int32_t* bsk_noise,
                         const u64* bsk_mask, const int32_t* ksk_mask, const int32_t* ksk_noise, u64* h_words,
                         int32_t* h_ksk) {
    const int n = c->p.n, N = c->p.N, k = c->p.k, kN = k * N;
    for (int i = 0; i < n; i++)
        if (lwe_s[i] != 0 && lwe_s[i] != 1) throw std::invalid_argument("LWE secret must be binary");
    for (int i = 0; i < kN; i++)
        if (rlwe_s[i] != 0 && rlwe_s[i] != 1) throw std::invalid_argument("RLWE secret must be binary");
    DeviceScratch scratch;
    const KeygenSamples d = alloc_samples(c, scratch);
    ck(cudaMemcpy(d.lwe_s, lwe_s, n * sizeof(int32_t), cudaMemcpyHostToDevice), "upload keygen");
    ck(cudaMemcpy(d.rlwe_s, rlwe_s, kN * sizeof(int32_t), cudaMemcpyHostToDevice), "upload keygen");
    ck(cudaMemcpy(d.noise, bsk_noise, d.samples * N * sizeof(int32_t), cudaMemcpyHostToDevice), "upload keygen noise");
    ck(cudaMemcpy(d.mask, bsk_mask, d.samples * k * N * sizeof(u64), cudaMemcpyHostToDevice), "upload keygen masks");
    ck(cudaMemcpy(d.kmask, ksk_mask, d.ksk_samples * n * sizeof(int32_t), cudaMemcpyHostToDevice), "upload KSK masks");
    ck(cudaMemcpy(d.knoise, ksk_noise, d.ksk_samples * sizeof(int32_t), cudaMemcpyHostToDevice), "upload KSK noise");
    keygen_on_device(c, key, rlwe_s, d, h_words, h_ksk, scratch);
}

// The context's mod-q forward twiddles on the device, uploaded by the first caller.
const u64* ctx_qfwd(yg_ctx* c) {
    std::lock_guard<std::mutex> lk(c->qfwd_mu);
    if (!c->d_qfwd) {
        const size_t N = (size_t)c->p.N;
        u64* d = nullptr;
        ck(cudaMalloc(&d, 2 * N * sizeof(u64)), "cudaMalloc mod-q twiddles");
        if (cudaMemcpy(d, c->qtab->wf.data(), N * sizeof(u64), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d + N, c->qtab->wfp.data(), N * sizeof(u64), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(d);
            throw CudaError("upload mod-q twiddles");
        }
        c->d_qfwd = d;
    }
    return c->d_qfwd;
}

// Launch arguments of the NTT-domain RLWE encryption (buffers left to the caller):
// q^-1 mod 2^64 by Newton's iteration (each step doubles the correct low bits of an odd
// q's inverse, from 3 bits for inv = q) and 2^128 mod q.
yg::EncryptRlweArgs rlwe_encrypt_args(yg_ctx* c) {
    yg::EncryptRlweArgs a{};
    const u64 q = c->q;
    u64 inv = q;
    for (int i = 0; i < 6; i++) inv *= 2 - q * inv;
    const u64 r1 = (u64)(((u128)1 << 64) % q);
    const u64* tw = ctx_qfwd(c);
    a.wf = tw;
    a.wfp = tw + c->p.N;
    a.q = q;
    a.qinv = inv;
    a.r2 = mulmod(r1, r1, q);
    a.N = c->p.N;
    a.k = c->p.k;
    a.torus_bits = c->p.torus_bits;
    a.ctas = 2 * c->sm_count;
    return a;
}

// deserializeBskMP / deserialize(TrgswMPDft|TrlweDft|NttPolynomial)
// (yatfhe/src/ya_serializer.cpp:21-30,87-98,193-218,287-303): native-endian PODs.
struct Reader {
    FILE* f;
    std::string path;
    void raw(void* p, size_t n) {
        if (std::fread(p, 1, n, f) != n) throw std::runtime_error("short read in " + path);
    }
    int32_t i32() {
        int32_t v;
        raw(&v, 4);
        return v;
    }
    uint8_t b8() {
        uint8_t v;
        raw(&v, 1);
        return v;
    }
    void expect(int32_t want, const char* what) {
        const int32_t v = i32();
        if (v != want)
            throw std::runtime_error(path + ": " + what + " is " + std::to_string(v) + ", expected " +
                                     std::to_string(want));
    }
};

void read_trlwe_dft(Reader& r, u64* rows, int k, int N) {
    r.expect(k, "TrlweDft k");
    if (r.b8() != 1) throw std::runtime_error(r.path + ": TrlweDft without its mask polynomials");
    r.expect(N, "NttPolynomial N");
    r.raw(rows + (size_t)k * N, sizeof(u64) * N);
    r.expect(k, "TrlweDft a size");
    for (int p = 0; p < k; p++) {
        r.expect(N, "NttPolynomial N");
        r.raw(rows + (size_t)p * N, sizeof(u64) * N);
    }
}

std::vector<u64> read_bsk_file(const yg_params& p, const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    Reader r{f, path};
    const int n = p.n, N = p.N, k = p.k, L = p.l_approx;
    const size_t row = (size_t)(k + 1) * N, lvl = (size_t)(k + 1) * row;
    std::vector<u64> words((size_t)n * L * lvl);
    try {
        for (int i = 0; i < n; i++) {
            r.expect(L, "TrgswMPDft l");
            r.expect(k, "TrgswMPDft k");
            if (r.b8() != 0) throw std::runtime_error(std::string(path) + ": half (cPrime-only) keys are not GINX keys");
            r.expect(L, "c size");
            for (int l = 0; l < L; l++) {
                r.expect(k, "c[l] size");
                for (int rr = 0; rr < k; rr++) read_trlwe_dft(r, words.data() + ((size_t)i * L + l) * lvl + rr * row, k, N);
            }
            r.expect(L, "cPrime size");
            for (int l = 0; l < L; l++) read_trlwe_dft(r, words.data() + ((size_t)i * L + l) * lvl + (size_t)k * row, k, N);
        }
        r.expect(n, "key n");
        r.expect(1, "key group");
        r.b8();
    } catch (...) {
        std::fclose(f);
        throw;
    }
    std::fclose(f);
    return words;
}

// deserializeBskWWL24 (yatfhe/src/ya_serializer.cpp:231-246): n half TrgswMPDft (cPrime rows
// only, :193-218), the TrlevDft s2 (:107-115), then [int n][int group].  cprime out =
// [n][L][k+1][N], s2 out = [l][k+1][N].
int read_wwl24_file(const yg_params& p, const char* path, std::vector<u64>& cprime, std::vector<u64>& s2) {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    Reader r{f, path};
    const int n = p.n, N = p.N, k = p.k, L = p.l_approx;
    const size_t row = (size_t)(k + 1) * N;
    cprime.assign((size_t)n * L * row, 0);
    int Ls = 0;
    try {
        for (int i = 0; i < n; i++) {
            r.expect(L, "TrgswMPDft l");
            r.expect(k, "TrgswMPDft k");
            if (r.b8() != 1) throw std::runtime_error(std::string(path) + ": full TRGSW rows are not a WWL+24 key");
            r.expect(L, "cPrime size");
            for (int l = 0; l < L; l++) read_trlwe_dft(r, cprime.data() + ((size_t)i * L + l) * row, k, N);
        }
        Ls = r.i32();
        if (Ls < 1 || Ls > yg::kWwlMaxLevels) throw std::runtime_error(std::string(path) + ": s2 key levels out of range");
        r.expect(Ls, "TrlevDft size");
        s2.assign((size_t)Ls * row, 0);
        for (int l = 0; l < Ls; l++) read_trlwe_dft(r, s2.data() + (size_t)l * row, k, N);
        r.expect(n, "key n");
        r.expect(1, "key group");
    } catch (...) {
        std::fclose(f);
        throw;
    }
    std::fclose(f);
    return Ls;
}

// deserializeBskLazyPipeAlt (yatfhe/src/ya_serializer.cpp:462-481): the TrlevDft s2
// (`[int l][int l]` + l TrlweDft), n half TrgswMP (`[int L][int k][bool 1][int L]` + L Trlwe,
// :148-174; a Trlwe is `[int k][int N]`, b, `[int k]`, a_0..a_{k-1}, each a TorusPolynomial
// `[int N]` + N Torus words, :33-42,65-74), then `[int level][int group]`.  Torus words are
// int32 in the reference's 32-bit build, int64 in its 56-bit build.
int read_lazy_file(const yg_params& p, const char* path, std::vector<int64_t>& cprime, std::vector<u64>& s2) {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    Reader r{f, path};
    const int n = p.n, N = p.N, k = p.k, L = p.l_approx;
    const size_t row = (size_t)(k + 1) * N;
    auto torus_poly = [&](int64_t* dst) {
        r.expect(N, "TorusPolynomial N");
        if (p.torus_bits == 32) {
            std::vector<int32_t> w(N);
            r.raw(w.data(), 4 * (size_t)N);
            for (int j = 0; j < N; j++) dst[j] = w[j];
        } else {
            r.raw(dst, 8 * (size_t)N);
        }
    };
    int Ls = 0;
    try {
        Ls = r.i32();
        if (Ls < 1 || Ls > yg::kLazyMaxLevels) throw std::runtime_error(std::string(path) + ": s2 key levels out of range");
        r.expect(Ls, "TrlevDft size");
        s2.assign((size_t)Ls * row, 0);
        for (int l = 0; l < Ls; l++) read_trlwe_dft(r, s2.data() + (size_t)l * row, k, N);
        cprime.assign((size_t)n * L * row, 0);
        for (int i = 0; i < n; i++) {
            r.expect(L, "TrgswMP l");
            r.expect(k, "TrgswMP k");
            if (r.b8() != 1) throw std::runtime_error(std::string(path) + ": full TRGSW rows are not a lazy key");
            r.expect(L, "cPrime size");
            for (int l = 0; l < L; l++) {
                int64_t* t = cprime.data() + ((size_t)i * L + l) * row;
                r.expect(k, "Trlwe k");
                r.expect(N, "Trlwe N");
                torus_poly(t + (size_t)k * N);
                r.expect(k, "Trlwe a size");
                for (int a = 0; a < k; a++) torus_poly(t + (size_t)a * N);
            }
        }
        r.expect(L, "key level");
        r.expect(1, "key group");
    } catch (...) {
        std::fclose(f);
        throw;
    }
    std::fclose(f);
    return Ls;
}

// The group blind rotation's launch arguments for a context and group key (buffers and count
// left empty).
yg::GroupBrArgs group_args(const yg_ctx* c, const yg_key* key) {
    yg::GroupBrArgs a{};
    const int N = c->p.N;
    const u64 q = c->q;
    const u64* tab = key->d_group_tab;
    a.key = key->d_group;
    a.wi = tab;
    a.wip = tab + N;
    a.wf = tab + 2 * (size_t)N;
    a.wfp = tab + 3 * (size_t)N;
    a.psi_m = tab + 4 * (size_t)N;
    a.slot_exp = tab + 6 * (size_t)N;
    a.q = q;
    u64 inv = q;
    for (int i = 0; i < 6; i++) inv *= 2 - q * inv;
    a.qinv = inv;
    a.post = mulmod(c->qtab->ninv, (u64)(((u128)1 << 64) % q), q);
    a.postp = (u64)(((u128)a.post << 64) / q);
    a.n = c->p.n;
    a.N = N;
    a.L = c->p.l_approx;
    a.l_full = key->group_levels;
    a.group = key->group;
    a.radix_bits = c->p.radix_bits;
    a.torus_bits = c->p.torus_bits;
    return a;
}

// The lazy blind rotation's launch arguments for a context and lazy key (buffers and count
// left empty).
yg::LazyBrArgs lazy_args(const yg_ctx* c, const yg_key* key) {
    yg::LazyBrArgs a{};
    const int N = c->p.N, T = c->p.torus_bits, rb = c->p.radix_bits, Ls = key->lazy_ls;
    const u64 q = c->q;
    const u64* tab = key->d_lazy_tab;
    a.cprime = key->d_lazy_cprime;
    a.wi = tab;
    a.wip = tab + N;
    a.wf = tab + 2 * (size_t)N;
    a.wfp = tab + 3 * (size_t)N;
    a.s2 = tab + 4 * (size_t)N;
    a.s2p = a.s2 + (size_t)Ls * 2 * N;
    a.q = q;
    u64 inv = q;  // Newton: each step doubles the bits of q^-1 mod 2^64 that are right
    for (int i = 0; i < 6; i++) inv *= 2 - q * inv;
    a.qinv = inv;
    a.post = mulmod(c->qtab->ninv, (u64)(((u128)1 << 64) % q), q);
    a.postp = (u64)(((u128)a.post << 64) / q);
    for (int gl = 0; gl < Ls; gl++) {
        const int64_t g = sext_host((int64_t)1 << (T - (gl + 1) * rb), T);
        a.recomp[gl] = g < 0 ? (u64)(g + (int64_t)q) : (u64)g;
        a.recompp[gl] = (u64)(((u128)a.recomp[gl] << 64) / q);
    }
    a.n = c->p.n;
    a.N = N;
    a.L = c->p.l_approx;
    a.Ls = Ls;
    a.radix_bits = rb;
    a.torus_bits = T;
    return a;
}

}  // namespace

yg::BrArgs yg::br_args(const yg_ctx* c, const yg_key* key) {
    yg::BrArgs a{};
    a.key = key ? reinterpret_cast<const uint4*>(key->d_bsk) : nullptr;
    a.n = c->p.n;
    a.steps = c->p.n;
    a.L = c->p.l_approx;
    a.radix_bits = c->p.radix_bits;
    for (int ci = 0; ci < yg::kChannels; ci++) a.ch[ci] = c->ch[ci];
    a.crt = c->crt;
    a.tw16 = c->d_tw16;
    a.per_cta = c->per_cta;
    a.layout = c->layout;
    a.grid = c->ctas_per_sm > 0 ? c->ctas_per_sm * c->sm_count : 0;
    return a;
}

yg::BrArgs yg::br_args(const yg_ctx* c, const yg_key* key, int count) {
    yg::BrArgs a = br_args(c, key);
    a.count = count;
    if (!c->launch_set && count <= c->latency_max) {
        a.layout = yg::kLayoutChannelCluster;
        a.per_cta = 1;
        a.grid = 0;
    }
    return a;
}

int yg::check_key(const yg_ctx* c, const yg_key* k, bool need_bsk, bool need_ksk, bool lazy_ok) {
    if (!c || !k) return set_err(YG_ERR_INVALID, "null context or key");
    if (k->ctx != c) return set_err(YG_ERR_INVALID, "key belongs to another context");
    if (need_bsk && (k->lazy() || k->grouped()) && !lazy_ok)
        return set_err(YG_ERR_INVALID,
                       "lazy and group keys run through yg_pbs, yg_pbs_host, yg_blind_rotate and yg_blind_rotate_extract");
    if (need_bsk && !k->d_bsk && !k->lazy() && !k->grouped())
        return set_err(YG_ERR_STATE, "key has no bootstrapping key");
    if (need_ksk && !k->d_ksk) return set_err(YG_ERR_STATE, "key has no key-switching key (yg_key_set_ksk)");
    return YG_OK;
}

namespace {

using yg::br_args;
using yg::check_key;

// yg_pbs_host pipelines batches of at least 4 x kPipelineChunk ciphertexts in 4 chunks.
constexpr int kPipelineChunk = 4096;

int do_pbs(yg_ctx* c, const yg_key* key, const int32_t* d_in, int32_t* d_out, int count, const int64_t* d_lut,
           cudaStream_t s) {
    const int N = c->p.N, kN = c->p.k * N;
    int32_t* big = nullptr;
    ck(cudaMallocAsync(&big, (size_t)count * (kN + 1) * sizeof(int32_t), s), "cudaMallocAsync extract buffer");
    int rc;
    if (key->grouped()) {
        yg::GroupBrArgs a = group_args(c, key);
        a.lwe_in = d_in;
        a.lut = d_lut;
        a.big_out = big;
        a.count = count;
        rc = yg::launch_group_blind_rotate(a, s);
    } else if (key->lazy()) {
        yg::LazyBrArgs a = lazy_args(c, key);
        a.lwe_in = d_in;
        a.lut = d_lut;
        a.big_out = big;
        a.count = count;
        rc = yg::launch_lazy_blind_rotate(a, s);
    } else {
        yg::BrArgs a = br_args(c, key, count);
        a.lwe_in = d_in;
        a.lut = d_lut;
        a.big_out = big;
        rc = yg::launch_blind_rotate(c->logN, c->p.torus_bits, a, s);
    }
    if (rc == 0) {
        yg::KsArgs k{big, key->d_ksk, d_out, count, kN, c->p.n, c->p.ks_level, c->p.ks_radix_bits};
        rc = yg::launch_keyswitch(k, s);
    }
    cudaError_t e = cudaFreeAsync(big, s);
    yg::check_launch(rc, "bootstrap launch");
    ck(e, "cudaFreeAsync");
    return YG_OK;
}

}  // namespace

namespace yg {

LazyBrArgs lazy_launch_args(const yg_ctx* c, const yg_key* key) { return lazy_args(c, key); }

size_t lazy_cprime_bytes(const yg_params& p) {
    return (size_t)p.n * p.l_approx * (p.k + 1) * p.N * (p.torus_bits == 32 ? 4 : 8);
}

size_t lazy_tab_words(const yg_params& p, int Ls) { return 4 * (size_t)p.N + 2 * (size_t)Ls * (p.k + 1) * p.N; }

LazyKeyRef lazy_key_ref(const yg_params& p, const void* cprime, const uint64_t* tab, int Ls) {
    const uint64_t* s2 = tab + 4 * (size_t)p.N;
    return LazyKeyRef{cprime, s2, s2 + (size_t)Ls * (p.k + 1) * p.N};
}

}  // namespace yg

extern "C" {

const char* yg_last_error(void) { return yg::last_error_slot().c_str(); }

int yg_ctx_create(const yg_params* params, int device, yg_ctx** out) {
    if (!params || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        validate(*params);
        DeviceGuard g(device);
        auto c = std::make_unique<yg_ctx>();
        c->p = *params;
        c->device = device;
        c->logN = params->N == 1024 ? 10 : 11;
        c->ps = yg::prime_set_for(params->torus_bits);
        c->q = params->torus_bits == 32 ? 562941363486721ULL : 1945555039024054273ULL;
        c->qtab = std::make_shared<QTables>(params->N, c->q);
        ck(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device), "SM count");
        ctx_init_tables(c.get());
        // small batches run in the channel-cluster layout until yg_ctx_set_launch is called:
        // up to two waves of its six-CTA clusters
        if (c->d_tw16 && yg::br_ctas_per_sm(c->logN, c->p.torus_bits, c->p.n, c->p.l_approx, 1,
                                            yg::kLayoutChannelCluster) >= 1) {
            const int clusters = yg::cluster6_max_clusters(c->p.n, c->p.l_approx);
            c->latency_max = 2 * (clusters > 0 ? clusters : c->sm_count / 6);
        }
        *out = c.release();
        return YG_OK;
    });
}

void yg_ctx_destroy(yg_ctx* ctx) {
    if (!ctx) return;
    if (ctx->d_tw) cudaFree(ctx->d_tw);
    if (ctx->d_tw16) cudaFree(ctx->d_tw16);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->d_qfwd) cudaFree(ctx->d_qfwd);
    delete ctx;
}

int yg_key_upload_bsk_ntt(yg_ctx* ctx, const uint64_t* h_bsk_ntt, yg_key** out) {
    if (!ctx || !h_bsk_ntt || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        auto k = std::make_unique<yg_key>();
        k->ctx = ctx;
        try {
            upload_bsk(ctx, k.get(), h_bsk_ntt);
        } catch (...) {
            if (k->d_bsk) cudaFree(k->d_bsk);
            k->d_bsk = nullptr;
            throw;
        }
        *out = k.release();
        return YG_OK;
    });
}

int yg_key_load_bsk_file(yg_ctx* ctx, const char* path, yg_key** out) {
    if (!ctx || !path || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        std::vector<u64> words = read_bsk_file(ctx->p, path);
        return yg_key_upload_bsk_ntt(ctx, words.data(), out);
    });
}

int yg_key_upload_wwl24_ntt(yg_ctx* ctx, const uint64_t* h_cprime, const uint64_t* h_s2, int s2_levels, yg_key** out) {
    if (!ctx || !h_cprime || !h_s2 || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        auto k = std::make_unique<yg_key>();
        k->ctx = ctx;
        try {
            upload_wwl24(ctx, k.get(), h_cprime, h_s2, s2_levels);
        } catch (...) {
            if (k->d_bsk) cudaFree(k->d_bsk);
            k->d_bsk = nullptr;
            throw;
        }
        *out = k.release();
        return YG_OK;
    });
}

int yg_key_load_wwl24_file(yg_ctx* ctx, const char* path, yg_key** out) {
    if (!ctx || !path || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        std::vector<u64> cprime, s2;
        const int levels = read_wwl24_file(ctx->p, path, cprime, s2);
        return yg_key_upload_wwl24_ntt(ctx, cprime.data(), s2.data(), levels, out);
    });
}

int yg_key_upload_lazy(yg_ctx* ctx, const int64_t* h_cprime, const uint64_t* h_s2, int s2_levels, yg_key** out) {
    if (!ctx || !h_cprime || !h_s2 || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        auto k = std::make_unique<yg_key>();
        k->ctx = ctx;
        try {
            upload_lazy(ctx, k.get(), h_cprime, h_s2, s2_levels);
        } catch (...) {
            if (k->d_lazy_cprime) cudaFree(k->d_lazy_cprime);
            if (k->d_lazy_tab) cudaFree(k->d_lazy_tab);
            k->d_lazy_cprime = nullptr;
            k->d_lazy_tab = nullptr;
            throw;
        }
        *out = k.release();
        return YG_OK;
    });
}

int yg_key_upload_group(yg_ctx* ctx, const uint64_t* h_words, int group, int key_levels, yg_key** out) {
    if (!ctx || !h_words || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        auto k = std::make_unique<yg_key>();
        k->ctx = ctx;
        try {
            upload_group(ctx, k.get(), h_words, group, key_levels);
        } catch (...) {
            if (k->d_group) cudaFree(k->d_group);
            if (k->d_group_tab) cudaFree(k->d_group_tab);
            k->d_group = nullptr;
            k->d_group_tab = nullptr;
            throw;
        }
        *out = k.release();
        return YG_OK;
    });
}

int yg_key_load_lazy_file(yg_ctx* ctx, const char* path, yg_key** out) {
    if (!ctx || !path || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        std::vector<int64_t> cprime;
        std::vector<u64> s2;
        const int levels = read_lazy_file(ctx->p, path, cprime, s2);
        return yg_key_upload_lazy(ctx, cprime.data(), s2.data(), levels, out);
    });
}

int yg_keygen_from_samples(yg_ctx* ctx, const int32_t* h_lwe_s, const int32_t* h_rlwe_s, const int32_t* h_bsk_noise,
                           const uint64_t* h_bsk_mask, const int32_t* h_ksk_mask, const int32_t* h_ksk_noise,
                           uint64_t* h_bsk_words, int32_t* h_ksk, yg_key** out) {
    if (!ctx || !h_lwe_s || !h_rlwe_s || !h_bsk_noise || !h_bsk_mask || !h_ksk_mask || !h_ksk_noise || !out)
        return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        auto k = std::make_unique<yg_key>();
        k->ctx = ctx;
        try {
            keygen_from_samples(ctx, k.get(), h_lwe_s, h_rlwe_s, h_bsk_noise, h_bsk_mask, h_ksk_mask, h_ksk_noise,
                                h_bsk_words, h_ksk);
        } catch (...) {
            if (k->d_bsk) cudaFree(k->d_bsk);
            if (k->d_ksk) cudaFree(k->d_ksk);
            k->d_bsk = nullptr;
            k->d_ksk = nullptr;
            throw;
        }
        *out = k.release();
        return YG_OK;
    });
}

int yg_draw_keygen_samples(yg_ctx* ctx, uint64_t seed, int lwe_noise_b, int rlwe_noise_b, int32_t* h_lwe_s,
                           int32_t* h_rlwe_s, int32_t* h_bsk_noise, uint64_t* h_bsk_mask, int32_t* h_ksk_mask,
                           int32_t* h_ksk_noise) {
    if (!ctx || !h_lwe_s || !h_rlwe_s || !h_bsk_noise || !h_bsk_mask || !h_ksk_mask || !h_ksk_noise)
        return set_err(YG_ERR_INVALID, "null argument");
    return guarded([&] {
        DeviceGuard g(ctx->device);
        DeviceScratch scratch;
        const KeygenSamples d = alloc_samples(ctx, scratch);
        draw_keygen_samples(ctx, seed, lwe_noise_b, rlwe_noise_b, d);
        const int n = ctx->p.n, N = ctx->p.N, k = ctx->p.k;
        ck(cudaMemcpy(h_lwe_s, d.lwe_s, n * sizeof(int32_t), cudaMemcpyDeviceToHost), "download");
        ck(cudaMemcpy(h_rlwe_s, d.rlwe_s, (size_t)k * N * sizeof(int32_t), cudaMemcpyDeviceToHost), "download");
        ck(cudaMemcpy(h_bsk_noise, d.noise, d.samples * N * sizeof(int32_t), cudaMemcpyDeviceToHost), "download");
        ck(cudaMemcpy(h_bsk_mask, d.mask, d.samples * k * N * sizeof(u64), cudaMemcpyDeviceToHost), "download");
        ck(cudaMemcpy(h_ksk_mask, d.kmask, d.ksk_samples * n * sizeof(int32_t), cudaMemcpyDeviceToHost), "download");
        ck(cudaMemcpy(h_ksk_noise, d.knoise, d.ksk_samples * sizeof(int32_t), cudaMemcpyDeviceToHost), "download");
        return YG_OK;
    });
}

int yg_keygen(yg_ctx* ctx, uint64_t seed, int lwe_noise_b, int rlwe_noise_b, int32_t* h_lwe_s, int32_t* h_rlwe_s,
              yg_key** out) {
    if (!ctx || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        auto k = std::make_unique<yg_key>();
        k->ctx = ctx;
        try {
            DeviceScratch scratch;
            const KeygenSamples d = alloc_samples(ctx, scratch);
            draw_keygen_samples(ctx, seed, lwe_noise_b, rlwe_noise_b, d);
            const int n = ctx->p.n, kN = ctx->p.k * ctx->p.N;
            std::vector<int32_t> lwe_s(n), rlwe_s(kN);
            ck(cudaMemcpy(lwe_s.data(), d.lwe_s, n * sizeof(int32_t), cudaMemcpyDeviceToHost), "download secret");
            ck(cudaMemcpy(rlwe_s.data(), d.rlwe_s, kN * sizeof(int32_t), cudaMemcpyDeviceToHost), "download secret");
            keygen_on_device(ctx, k.get(), rlwe_s.data(), d, nullptr, nullptr, scratch);
            if (h_lwe_s) std::copy(lwe_s.begin(), lwe_s.end(), h_lwe_s);
            if (h_rlwe_s) std::copy(rlwe_s.begin(), rlwe_s.end(), h_rlwe_s);
        } catch (...) {
            if (k->d_bsk) cudaFree(k->d_bsk);
            if (k->d_ksk) cudaFree(k->d_ksk);
            k->d_bsk = nullptr;
            k->d_ksk = nullptr;
            throw;
        }
        *out = k.release();
        return YG_OK;
    });
}

int yg_encrypt_lwe(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, int count, uint64_t seed, uint32_t call,
                   int lwe_noise_b, int32_t* d_out, void* stream) {
    if (!ctx || count < 0 || (count > 0 && (!d_s || !d_mu || !d_out)) || lwe_noise_b < 0 || lwe_noise_b > 30)
        return set_err(YG_ERR_INVALID, "yg_encrypt_lwe: bad arguments");
    if (count == 0) return YG_OK;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        yg::EncryptArgs a{d_s, d_mu, nullptr, nullptr, d_out, seed, kDomEncrypt, call, count, ctx->p.n, lwe_noise_b};
        yg::check_launch(yg::launch_encrypt_lwe(a, stream), "encrypt launch");
        return YG_OK;
    });
}

int yg_encrypt_lwe_from_samples(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, const int32_t* d_mask,
                                const int32_t* d_noise, int count, int32_t* d_out, void* stream) {
    if (!ctx || count < 0 || (count > 0 && (!d_s || !d_mu || !d_mask || !d_noise || !d_out)))
        return set_err(YG_ERR_INVALID, "yg_encrypt_lwe_from_samples: bad arguments");
    if (count == 0) return YG_OK;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        yg::EncryptArgs a{d_s, d_mu, d_mask, d_noise, d_out, 0, 0, 0, count, ctx->p.n, 0};
        yg::check_launch(yg::launch_encrypt_lwe(a, stream), "encrypt launch");
        return YG_OK;
    });
}

int yg_encrypt_rlwe_ntt(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, int count, uint64_t seed, uint32_t call,
                        int rlwe_noise_b, uint64_t* d_out, void* stream) {
    if (!ctx || count < 0 || (count > 0 && (!d_s || !d_mu || !d_out)) || rlwe_noise_b < 0 || rlwe_noise_b > 30)
        return set_err(YG_ERR_INVALID, "yg_encrypt_rlwe_ntt: bad arguments");
    if (count == 0) return YG_OK;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        yg::EncryptRlweArgs a = rlwe_encrypt_args(ctx);
        const cudaStream_t st = (cudaStream_t)stream;
        const size_t N = (size_t)ctx->p.N, k = (size_t)ctx->p.k;
        int32_t* noise = nullptr;
        u64* mask = nullptr;
        ck(cudaMallocAsync((void**)&noise, count * N * sizeof(int32_t), st), "cudaMallocAsync noise");
        if (cudaMallocAsync((void**)&mask, count * k * N * sizeof(u64), st) != cudaSuccess) {
            cudaFreeAsync(noise, st);
            throw CudaError("cudaMallocAsync masks");
        }
        yg::DrawArgs dn{};
        dn.out_i32 = noise;
        dn.count = count * N;
        dn.seed = seed;
        dn.domain = kDomEncrypt + 1;
        dn.stream = call;
        dn.kind = yg::kDrawTUniform;
        dn.b = rlwe_noise_b;
        dn.per_block = 8;
        yg::DrawArgs dm{};
        dm.out_u64 = mask;
        dm.count = count * k * N;
        dm.seed = seed;
        dm.q = ctx->q;
        dm.domain = kDomEncrypt + 2;
        dm.stream = call;
        dm.kind = yg::kDrawModQ;
        dm.per_block = 4;
        a.s = d_s;
        a.mu = d_mu;
        a.noise = noise;
        a.mask = mask;
        a.out = d_out;
        a.count = count;
        const int rc = (yg::launch_draw(dn, stream) || yg::launch_draw(dm, stream) ||
                        yg::launch_encrypt_rlwe_ntt(a, stream)) ? -1 : 0;
        cudaFreeAsync(mask, st);
        cudaFreeAsync(noise, st);
        yg::check_launch(rc, "RLWE encryption launch");
        return YG_OK;
    });
}

int yg_encrypt_rlwe_ntt_from_samples(yg_ctx* ctx, const int32_t* d_s, const int64_t* d_mu, const uint64_t* d_mask,
                                     const int32_t* d_noise, int count, uint64_t* d_out, void* stream) {
    if (!ctx || count < 0 || (count > 0 && (!d_s || !d_mu || !d_mask || !d_noise || !d_out)))
        return set_err(YG_ERR_INVALID, "yg_encrypt_rlwe_ntt_from_samples: bad arguments");
    if (count == 0) return YG_OK;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        yg::EncryptRlweArgs a = rlwe_encrypt_args(ctx);
        const cudaStream_t st = (cudaStream_t)stream;
        int* bad = nullptr;
        ck(cudaMallocAsync((void**)&bad, sizeof(int), st), "cudaMallocAsync flag");
        a.s = d_s;
        a.mu = d_mu;
        a.noise = d_noise;
        a.mask = d_mask;
        a.out = d_out;
        a.count = count;
        a.bad = bad;
        int h_bad = 0;
        cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(int), st);
        const int rc = e == cudaSuccess ? yg::launch_encrypt_rlwe_ntt(a, stream) : -1;
        if (rc == 0) e = cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaFreeAsync(bad, st);
        yg::check_launch(rc, "RLWE encryption launch");
        ck(e, "RLWE encryption flag");
        ck(cudaStreamSynchronize(st), "RLWE encryption");
        if (h_bad) return set_err(YG_ERR_INVALID, "RLWE mask word not reduced mod q");
        return YG_OK;
    });
}

// ------------------------------------------------------------------ approximate CRT

struct yg_crt_key {
    int device = 0, n = 0, N = 0, logN = 0, sm_count = 0;
    uint2* d_tw = nullptr;        // [N forward | 2N inverse] tables of 2^24 - 2^14 + 1
    uint32_t* d_key = nullptr;    // [n][d][dh][2 rows] key blocks (key_block_words(N) each)
    size_t key_bytes = 0;
    yg::Chan ch{};
    yg::CrtBrArgs args{};         // constants of the rotation (buffers and count left empty)
};

namespace {

int64_t inv_small(int64_t a, int64_t m) {
    a %= m;
    if (a < 0) a += m;
    for (int64_t x = 1; x < m; x++)
        if (a * x % m == 1) return x;
    throw std::invalid_argument("not invertible");
}

}  // namespace

int yg_crt_key_upload(int device, int n, int N, const int8_t* h_bsk8, yg_crt_key** out) {
    if (!h_bsk8 || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n < 1 || n > 4096 || (N != 1024 && N != 2048)) return set_err(YG_ERR_INVALID, "ApproxCRT key: 1 <= n <= 4096, N = 1024 or 2048");
    return guarded([&] {
        DeviceGuard g(device);
        auto k = std::make_unique<yg_crt_key>();
        k->device = device;
        k->n = n;
        k->N = N;
        k->logN = N == 1024 ? 10 : 11;
        ck(cudaDeviceGetAttribute(&k->sm_count, cudaDevAttrMultiProcessorCount, device), "device attribute");
        const size_t rows = (size_t)n * yg::kCrtD * yg::kCrtDh * 2;
        const size_t bytes8 = rows * 2 * N;
        for (size_t e = 0; e < bytes8; e++) {
            const int v = h_bsk8[e];
            if (v < -125 || v > 125) throw std::invalid_argument("ApproxCRT key residue outside [-125, 125]");
        }
        // the transform tables of 2^24 - 2^14 + 1 (the Gentleman-Sande inverse at both N)
        const uint32_t p = yg::kMod24;
        std::vector<uint2> tw((size_t)3 * N), heads((size_t)yg::kChannels * 2 * 32);
        team_tables(p, N, k->logN, false, tw.data(), heads.data());
        for (int ci = 1; ci < yg::kChannels; ci++) std::copy(heads.begin(), heads.begin() + 64, heads.begin() + ci * 64);
        try {
            ck(cudaMalloc(&k->d_tw, tw.size() * sizeof(uint2)), "cudaMalloc twiddles");
            ck(cudaMemcpy(k->d_tw, tw.data(), tw.size() * sizeof(uint2), cudaMemcpyHostToDevice), "upload twiddles");
            if (yg::set_crt_twiddle_heads(k->logN, heads.data()) != 0) ck(cudaGetLastError(), "upload twiddle heads");
            k->ch = yg::Chan{p, 2 * p, neg_pinv32(p), 0, k->d_tw, k->d_tw + N};
            k->key_bytes = rows * yg::key_block_words(N) * sizeof(uint32_t);
            ck(cudaMalloc(&k->d_key, k->key_bytes), "cudaMalloc ApproxCRT key");
            DeviceScratch scratch;
            int8_t* d8 = scratch.alloc<int8_t>(bytes8, "cudaMalloc key upload");
            ck(cudaMemcpy(d8, h_bsk8, bytes8, cudaMemcpyHostToDevice), "upload ApproxCRT key");
            const uint32_t sc = conv_scale_for(p, N);
            yg::CrtKeyConvArgs ka{d8, k->d_key, k->ch, sc, shoup32(sc, p), (int)rows};
            yg::check_launch(yg::launch_crt_keyconv(k->logN, ka, nullptr), "ApproxCRT key conversion");
            ck(cudaDeviceSynchronize(), "ApproxCRT key conversion");
        } catch (...) {
            if (k->d_tw) cudaFree(k->d_tw);
            if (k->d_key) cudaFree(k->d_key);
            throw;
        }
        // initYatfhe's constants of the CRT (yatfhe/src/initializer.cpp:31-83): taoU and
        // taoUInv of the low primes, z_d = (Q / q_d) ((Q / q_d)^-1 mod q_d)
        const int64_t q[yg::kCrtD] = {251, 241, 239, 233};
        const int64_t qLow = q[2] * q[3], Q = q[0] * q[1] * qLow;
        yg::CrtBrArgs& a = k->args;
        for (int d = 0; d < yg::kCrtD; d++) {
            a.tao_u[d] = a.tao_u_inv[d] = 1;
            if (d >= yg::kCrtDh) {
                a.tao_u[d] = inv_small(qLow / q[d], q[d]);
                a.tao_u_inv[d] = (qLow / q[d]) % q[d];
            }
            a.z[d] = (Q / q[d]) * inv_small(Q / q[d], q[d]);
        }
        a.q_crt = Q;
        a.key = k->d_key;
        a.ch = k->ch;
        a.n = n;
        *out = k.release();
        return YG_OK;
    });
}

int yg_crt_blind_rotate(yg_crt_key* key, const int32_t* d_acc_in, const int32_t* d_rot, int count, int32_t* d_acc_out,
                        void* stream) {
    if (!key || count < 0 || (count > 0 && (!d_acc_in || !d_rot || !d_acc_out)))
        return set_err(YG_ERR_INVALID, "yg_crt_blind_rotate: bad arguments");
    if (count == 0) return YG_OK;
    return guarded([&] {
        DeviceGuard g(key->device);
        yg::CrtBrArgs a = key->args;
        a.acc_in = d_acc_in;
        a.rot = d_rot;
        a.acc_out = d_acc_out;
        a.count = count;
        int per_sm = 0;
        ck(yg::crt_blind_rotate_ctas_per_sm(key->logN, key->n, &per_sm) == 0 ? cudaSuccess : cudaErrorInvalidValue,
           "ApproxCRT occupancy");
        if (per_sm < 1) throw std::invalid_argument("ApproxCRT blind rotation does not fit an SM");
        const int grid = std::min(count, per_sm * key->sm_count);
        yg::check_launch(yg::launch_crt_blind_rotate(key->logN, a, grid, stream), "ApproxCRT blind rotation");
        return YG_OK;
    });
}

size_t yg_crt_key_device_bytes(const yg_crt_key* key) { return key ? key->key_bytes : 0; }

void yg_crt_key_destroy(yg_crt_key* key) {
    if (!key) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(key->device);
    if (key->d_tw) cudaFree(key->d_tw);
    if (key->d_key) cudaFree(key->d_key);
    if (prev >= 0) cudaSetDevice(prev);
    delete key;
}

int yg_key_set_ksk(yg_key* key, const int32_t* h_ksk) {
    if (!key || !h_ksk) return set_err(YG_ERR_INVALID, "null argument");
    return guarded([&] {
        const yg_params& p = key->ctx->p;
        DeviceGuard g(key->ctx->device);
        const size_t bytes = (size_t)p.k * p.N * p.ks_level * (p.n + 1) * sizeof(int32_t);
        if (!key->d_ksk) {
            ck(cudaMalloc(&key->d_ksk, bytes), "cudaMalloc ksk");
            key->ksk_bytes = bytes;
        }
        ck(cudaMemcpy(key->d_ksk, h_ksk, bytes, cudaMemcpyHostToDevice), "upload ksk");
        return YG_OK;
    });
}

void yg_key_destroy(yg_key* key) {
    if (!key) return;
    if (key->d_bsk) cudaFree(key->d_bsk);
    if (key->d_ksk) cudaFree(key->d_ksk);
    if (key->d_lazy_cprime) cudaFree(key->d_lazy_cprime);
    if (key->d_lazy_tab) cudaFree(key->d_lazy_tab);
    if (key->d_group) cudaFree(key->d_group);
    if (key->d_group_tab) cudaFree(key->d_group_tab);
    delete key;
}

size_t yg_key_device_bytes(const yg_key* key) { return key ? key->bsk_bytes + key->ksk_bytes : 0; }

int yg_pbs(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, int32_t* d_out, int count, const int64_t* d_lut,
           void* stream) {
    if (int rc = check_key(ctx, key, true, true, true)) return rc;
    if (count < 0 || (count > 0 && (!d_in || !d_out || !d_lut))) return set_err(YG_ERR_INVALID, "bad buffers");
    if (count == 0) return YG_OK;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        return do_pbs(ctx, key, d_in, d_out, count, d_lut, (cudaStream_t)stream);
    });
}

int yg_pbs_host(yg_ctx* ctx, const yg_key* key, const int32_t* h_in, int32_t* h_out, int count, const int64_t* h_lut,
                void* stream) {
    if (int rc = check_key(ctx, key, true, true, true)) return rc;
    if (count < 0 || (count > 0 && (!h_in || !h_out || !h_lut))) return set_err(YG_ERR_INVALID, "bad buffers");
    if (count == 0) return YG_OK;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        cudaStream_t s = (cudaStream_t)stream;
        const size_t n1 = (size_t)ctx->p.n + 1;
        const size_t lwe = (size_t)count * n1 * sizeof(int32_t);
        const size_t lut = (size_t)ctx->p.N * sizeof(int64_t);
        // large batches run as chunks alternating between the caller's stream and a side
        // stream, so one chunk's copies overlap another chunk's kernels
        const int chunks = count >= 4 * kPipelineChunk ? 4 : 1;
        cudaStream_t side = s;
        if (chunks > 1) {
            std::lock_guard<std::mutex> lk(ctx->side_mu);
            if (!ctx->side) ck(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking), "side stream");
            side = ctx->side;
        }
        char* d = nullptr;
        ck(cudaMallocAsync(&d, 2 * lwe + lut, s), "cudaMallocAsync io");
        int32_t* d_in = reinterpret_cast<int32_t*>(d);
        int32_t* d_out = reinterpret_cast<int32_t*>(d + lwe);
        int64_t* d_lut = reinterpret_cast<int64_t*>(d + 2 * lwe);
        cudaEvent_t ev[2] = {nullptr, nullptr};
        try {
            ck(cudaMemcpyAsync(d_lut, h_lut, lut, cudaMemcpyHostToDevice, s), "copy lut");
            if (chunks > 1) {
                for (auto& e : ev) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
                ck(cudaEventRecord(ev[0], s), "event");  // buffers allocated, LUT copied
                ck(cudaStreamWaitEvent(side, ev[0], 0), "wait");
            }
            for (int c = 0; c < chunks; c++) {
                const int begin = (int)((long long)count * c / chunks), end = (int)((long long)count * (c + 1) / chunks);
                cudaStream_t cs = c % 2 ? side : s;
                const size_t off = (size_t)begin * n1, bytes = (size_t)(end - begin) * n1 * sizeof(int32_t);
                ck(cudaMemcpyAsync(d_in + off, h_in + off, bytes, cudaMemcpyHostToDevice, cs), "copy in");
                do_pbs(ctx, key, d_in + off, d_out + off, end - begin, d_lut, cs);
                ck(cudaMemcpyAsync(h_out + off, d_out + off, bytes, cudaMemcpyDeviceToHost, cs), "copy out");
            }
            if (chunks > 1) {
                ck(cudaEventRecord(ev[1], side), "event");
                ck(cudaStreamWaitEvent(s, ev[1], 0), "wait");  // the buffers are freed after both
            }
        } catch (...) {
            if (chunks > 1) cudaStreamSynchronize(side);
            cudaFreeAsync(d, s);
            for (auto& e : ev)
                if (e) cudaEventDestroy(e);
            throw;
        }
        ck(cudaFreeAsync(d, s), "cudaFreeAsync io");
        ck(cudaStreamSynchronize(s), "bootstrap");
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        return YG_OK;
    });
}

int yg_blind_rotate(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, const int64_t* d_lut, int64_t* d_acc,
                    int count, int steps, void* stream) {
    if (int rc = check_key(ctx, key, true, false, true)) return rc;
    if (count < 0 || steps < 0 || steps > ctx->p.n) return set_err(YG_ERR_INVALID, "bad count or steps");
    if ((key->lazy() || key->grouped()) && steps != ctx->p.n)
        return set_err(YG_ERR_INVALID, "a lazy or group key runs the whole rotation: steps = n");
    if (count == 0) return YG_OK;
    if (!d_in || !d_lut || !d_acc) return set_err(YG_ERR_INVALID, "bad buffers");
    if (key->grouped()) {
        return guarded([&] {
            DeviceGuard g(ctx->device);
            yg::GroupBrArgs a = group_args(ctx, key);
            a.lwe_in = d_in;
            a.lut = d_lut;
            a.acc_out = d_acc;
            a.count = count;
            yg::check_launch(yg::launch_group_blind_rotate(a, stream), "group blind rotate launch");
            return YG_OK;
        });
    }
    if (key->lazy()) {
        return guarded([&] {
            DeviceGuard g(ctx->device);
            yg::LazyBrArgs a = lazy_args(ctx, key);
            a.lwe_in = d_in;
            a.lut = d_lut;
            a.acc_out = d_acc;
            a.count = count;
            yg::check_launch(yg::launch_lazy_blind_rotate(a, stream), "lazy blind rotate launch");
            return YG_OK;
        });
    }
    return guarded([&] {
        DeviceGuard g(ctx->device);
        yg::BrArgs a = br_args(ctx, key, count);
        a.lwe_in = d_in;
        a.lut = d_lut;
        a.acc_out = d_acc;
        a.steps = steps;
        yg::check_launch(yg::launch_blind_rotate(ctx->logN, ctx->p.torus_bits, a, stream), "blind rotate launch");
        return YG_OK;
    });
}

int yg_blind_rotate_extract(yg_ctx* ctx, const yg_key* key, const int32_t* d_in, const int64_t* d_lut,
                            int32_t* d_big, int count, void* stream) {
    if (int rc = check_key(ctx, key, true, false, true)) return rc;
    if (count < 0) return set_err(YG_ERR_INVALID, "bad count");
    if (count == 0) return YG_OK;
    if (!d_in || !d_lut || !d_big) return set_err(YG_ERR_INVALID, "bad buffers");
    if (key->grouped()) {
        return guarded([&] {
            DeviceGuard g(ctx->device);
            yg::GroupBrArgs a = group_args(ctx, key);
            a.lwe_in = d_in;
            a.lut = d_lut;
            a.big_out = d_big;
            a.count = count;
            yg::check_launch(yg::launch_group_blind_rotate(a, stream), "group blind rotate launch");
            return YG_OK;
        });
    }
    if (key->lazy()) {
        return guarded([&] {
            DeviceGuard g(ctx->device);
            yg::LazyBrArgs a = lazy_args(ctx, key);
            a.lwe_in = d_in;
            a.lut = d_lut;
            a.big_out = d_big;
            a.count = count;
            yg::check_launch(yg::launch_lazy_blind_rotate(a, stream), "lazy blind rotate launch");
            return YG_OK;
        });
    }
    return guarded([&] {
        DeviceGuard g(ctx->device);
        yg::BrArgs a = br_args(ctx, key, count);
        a.lwe_in = d_in;
        a.lut = d_lut;
        a.big_out = d_big;
        yg::check_launch(yg::launch_blind_rotate(ctx->logN, ctx->p.torus_bits, a, stream), "blind rotate launch");
        return YG_OK;
    });
}

int yg_blind_rotate_acc(yg_ctx* ctx, const yg_key* key, const int32_t* d_scaled, int64_t* d_acc, int count,
                        void* stream) {
    if (int rc = check_key(ctx, key, true, false, key && key->grouped())) return rc;
    if (count < 0) return set_err(YG_ERR_INVALID, "bad count");
    if (count == 0) return YG_OK;
    if (!d_scaled || !d_acc) return set_err(YG_ERR_INVALID, "bad buffers");
    if (key->grouped()) {
        return guarded([&] {
            DeviceGuard g(ctx->device);
            yg::GroupBrArgs a = group_args(ctx, key);
            a.scaled_in = d_scaled;
            a.acc_in = d_acc;
            a.acc_out = d_acc;
            a.count = count;
            yg::check_launch(yg::launch_group_blind_rotate(a, stream), "group blind rotate launch");
            return YG_OK;
        });
    }
    return guarded([&] {
        DeviceGuard g(ctx->device);
        yg::BrArgs a = br_args(ctx, key, count);
        a.scaled_in = d_scaled;
        a.acc_in = d_acc;
        a.acc_out = d_acc;
        yg::check_launch(yg::launch_blind_rotate(ctx->logN, ctx->p.torus_bits, a, stream), "blind rotate launch");
        return YG_OK;
    });
}

int yg_key_create_ksk_only(yg_ctx* ctx, yg_key** out) {
    if (!ctx || !out) return set_err(YG_ERR_INVALID, "null argument");
    *out = new (std::nothrow) yg_key();
    if (!*out) return set_err(YG_ERR_NOMEM, "host allocation failed");
    (*out)->ctx = ctx;
    return YG_OK;
}

int yg_keyswitch(yg_ctx* ctx, const yg_key* key, const int32_t* d_big, int32_t* d_out, int count, void* stream) {
    if (int rc = check_key(ctx, key, false, true)) return rc;
    if (count < 0) return set_err(YG_ERR_INVALID, "bad count");
    if (count == 0) return YG_OK;
    if (!d_big || !d_out) return set_err(YG_ERR_INVALID, "bad buffers");
    return guarded([&] {
        DeviceGuard g(ctx->device);
        const int kN = ctx->p.k * ctx->p.N;
        yg::KsArgs k{d_big, key->d_ksk, d_out, count, kN, ctx->p.n, ctx->p.ks_level, ctx->p.ks_radix_bits};
        yg::check_launch(yg::launch_keyswitch(k, stream), "keyswitch launch");
        return YG_OK;
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------------- plans

struct yg_plan {
    yg_ctx* ctx = nullptr;
    int count = 0;
    int grid = 0;
    int per_cta = 0;
    int layout = 0;
    const yg_key* key0 = nullptr;     // uniform batch: the one key
    const int64_t* lut0 = nullptr;    // uniform LUT
    const uint4** d_key_table = nullptr;
    int32_t* d_key_of = nullptr;
    const int64_t** d_lut_table = nullptr;
    int32_t* d_lut_of = nullptr;
    yg::KsTile* d_tiles = nullptr;
    int num_tiles = 0;
    int32_t* d_big = nullptr;
    // lazy ("OURS") keys: the lazy blind rotation, keys by table
    bool lazy = false;
    yg::LazyKeyRef* d_lazy_keys = nullptr;
    yg::LazyBrArgs lazy_tmpl{};
};

namespace {

void plan_free(yg_plan* p) {
    cudaFree(p->d_key_table);
    cudaFree(p->d_key_of);
    cudaFree(p->d_lut_table);
    cudaFree(p->d_lut_of);
    cudaFree(p->d_tiles);
    cudaFree(p->d_big);
    cudaFree(p->d_lazy_keys);
}

template <typename T>
T* upload_vec(const std::vector<T>& v, const char* what) {
    T* d = nullptr;
    ck(cudaMalloc(&d, std::max<size_t>(1, v.size()) * sizeof(T)), what);
    if (!v.empty()) ck(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), what);
    return d;
}

}  // namespace

extern "C" {

int yg_plan_create(yg_ctx* ctx, const yg_key* const* keys, int num_keys, const int32_t* h_key_ids,
                   const int64_t* const* d_luts, int num_luts, const int32_t* h_lut_ids, int count, yg_plan** out) {
    if (!ctx || !keys || num_keys < 1 || !d_luts || num_luts < 1 || count < 0 || !out)
        return set_err(YG_ERR_INVALID, "yg_plan_create: bad arguments");
    *out = nullptr;
    // one key family per plan: GINX rows (and keys derived into them), or lazy keys with the
    // same number of s2 levels
    for (int i = 0; i < num_keys; i++) {
        if (int rc = check_key(ctx, keys[i], true, true, true)) return rc;
        if (keys[i]->grouped()) return set_err(YG_ERR_INVALID, "yg_plan_create: group keys run through yg_pbs");
        if (keys[i]->lazy() != keys[0]->lazy() || keys[i]->lazy_ls != keys[0]->lazy_ls)
            return set_err(YG_ERR_INVALID, "yg_plan_create: a plan takes keys of one family (GINX or lazy)");
    }
    for (int i = 0; i < num_luts; i++)
        if (!d_luts[i]) return set_err(YG_ERR_INVALID, "yg_plan_create: null LUT");
    for (int c = 0; c < count; c++) {
        if (h_key_ids && (h_key_ids[c] < 0 || h_key_ids[c] >= num_keys))
            return set_err(YG_ERR_INVALID, "yg_plan_create: key index out of range");
        if (h_lut_ids && (h_lut_ids[c] < 0 || h_lut_ids[c] >= num_luts))
            return set_err(YG_ERR_INVALID, "yg_plan_create: LUT index out of range");
    }
    return guarded([&] {
        DeviceGuard g(ctx->device);
        auto p = std::make_unique<yg_plan>();
        p->ctx = ctx;
        p->count = count;
        p->key0 = keys[0];
        p->lut0 = d_luts[0];
        try {
            const bool multi_key = h_key_ids && num_keys > 1;
            p->lazy = keys[0]->lazy();
            if (p->lazy) p->lazy_tmpl = yg::lazy_launch_args(ctx, keys[0]);
            if (multi_key && p->lazy) {
                std::vector<yg::LazyKeyRef> table(num_keys);
                for (int i = 0; i < num_keys; i++)
                    table[i] = yg::lazy_key_ref(ctx->p, keys[i]->d_lazy_cprime, keys[i]->d_lazy_tab, keys[i]->lazy_ls);
                p->d_lazy_keys = upload_vec(table, "plan lazy key table");
            }
            if (multi_key) {
                std::vector<const uint4*> table(num_keys);
                for (int i = 0; i < num_keys; i++) table[i] = reinterpret_cast<const uint4*>(keys[i]->d_bsk);
                p->d_key_table = upload_vec(table, "plan key table");
                p->d_key_of = upload_vec(std::vector<int32_t>(h_key_ids, h_key_ids + count), "plan key index");
                std::vector<yg::KsTile> tiles;
                for (int c = 0; c < count;) {
                    int e = c + 1;
                    while (e < count && e - c < yg::kKsTileCts && h_key_ids[e] == h_key_ids[c]) e++;
                    tiles.push_back(yg::KsTile{c, e - c, keys[h_key_ids[c]]->d_ksk});
                    c = e;
                }
                p->num_tiles = (int)tiles.size();
                p->d_tiles = upload_vec(tiles, "plan key-switch tiles");
            }
            if (h_lut_ids && num_luts > 1) {
                p->d_lut_table = upload_vec(std::vector<const int64_t*>(d_luts, d_luts + num_luts), "plan LUT table");
                p->d_lut_of = upload_vec(std::vector<int32_t>(h_lut_ids, h_lut_ids + count), "plan LUT index");
            }
            const size_t big = (size_t)std::max(count, 1) * (ctx->p.k * ctx->p.N + 1) * sizeof(int32_t);
            ck(cudaMalloc(&p->d_big, big), "plan extract buffer");
        } catch (...) {
            plan_free(p.get());
            throw;
        }
        *out = p.release();
        return YG_OK;
    });
}

int yg_plan_set_launch(yg_plan* plan, int layout, int per_cta, int grid) {
    if (!plan || per_cta < 0 || grid < 0 ||
        (layout != YG_LAYOUT_CHANNEL && layout != YG_LAYOUT_CHANNEL_ROW && layout != YG_LAYOUT_ROW_CLUSTER &&
         layout != YG_LAYOUT_CHANNEL_CLUSTER))
        return set_err(YG_ERR_INVALID, "yg_plan_set_launch: bad arguments");
    if (per_cta > 0) {
        int fit = 0;
        if (int rc = yg_ctas_per_sm(plan->ctx, layout, per_cta, &fit)) return rc;
        if (fit < 1) return set_err(YG_ERR_INVALID, "yg_plan_set_launch: a CTA of that shape does not fit an SM");
    }
    plan->layout = layout;
    plan->per_cta = per_cta;
    plan->grid = grid;
    return YG_OK;
}

int yg_plan_run(yg_plan* plan, const int32_t* d_in, int32_t* d_out, void* stream) {
    if (!plan) return set_err(YG_ERR_INVALID, "null plan");
    if (plan->count == 0) return YG_OK;
    if (!d_in || !d_out) return set_err(YG_ERR_INVALID, "bad buffers");
    yg_ctx* ctx = plan->ctx;
    return guarded([&] {
        DeviceGuard g(ctx->device);
        const int kN = ctx->p.k * ctx->p.N;
        if (plan->lazy) {
            yg::LazyBrArgs a = plan->lazy_tmpl;
            a.lwe_in = d_in;
            a.lut = plan->lut0;
            a.keys = plan->d_lazy_keys;
            a.key_of = plan->d_lazy_keys ? plan->d_key_of : nullptr;
            a.lut_table = plan->d_lut_table;
            a.lut_of = plan->d_lut_of;
            a.big_out = plan->d_big;
            a.count = plan->count;
            yg::check_launch(yg::launch_lazy_blind_rotate(a, stream), "lazy blind rotate launch");
            yg::KsArgs k{plan->d_big, plan->key0->d_ksk, d_out, plan->count, kN, ctx->p.n, ctx->p.ks_level,
                         ctx->p.ks_radix_bits, plan->d_tiles, plan->num_tiles};
            yg::check_launch(yg::launch_keyswitch(k, stream), "keyswitch launch");
            return YG_OK;
        }
        yg::BrArgs a = br_args(ctx, plan->key0);
        a.lwe_in = d_in;
        a.lut = plan->lut0;
        a.key_table = plan->d_key_table;
        a.key_of = plan->d_key_of;
        a.lut_table = plan->d_lut_table;
        a.lut_of = plan->d_lut_of;
        a.big_out = plan->d_big;
        a.count = plan->count;
        if (plan->per_cta == 0 && !ctx->launch_set && plan->count <= ctx->latency_max) {
            a.layout = yg::kLayoutChannelCluster;  // the context's default for a small batch
            a.per_cta = 1;
            a.grid = 0;
        }
        if (plan->per_cta > 0) {
            a.per_cta = plan->per_cta;
            a.layout = plan->layout;
            a.grid = plan->grid;
        }
        yg::check_launch(yg::launch_blind_rotate(ctx->logN, ctx->p.torus_bits, a, stream), "blind rotate launch");
        yg::KsArgs k{plan->d_big, plan->key0->d_ksk, d_out, plan->count, kN, ctx->p.n, ctx->p.ks_level,
                     ctx->p.ks_radix_bits, plan->d_tiles, plan->num_tiles};
        yg::check_launch(yg::launch_keyswitch(k, stream), "keyswitch launch");
        return YG_OK;
    });
}

void yg_plan_destroy(yg_plan* plan) {
    if (!plan) return;
    DeviceGuard g(plan->ctx->device);
    plan_free(plan);
    delete plan;
}

int yg_ctas_per_sm(yg_ctx* ctx, int layout, int per_cta, int* out) {
    if (!ctx || !out) return set_err(YG_ERR_INVALID, "null argument");
    if (layout != YG_LAYOUT_CHANNEL && layout != YG_LAYOUT_CHANNEL_ROW && layout != YG_LAYOUT_ROW_CLUSTER &&
        layout != YG_LAYOUT_CHANNEL_CLUSTER)
        return set_err(YG_ERR_INVALID, "yg_ctas_per_sm: unknown layout");
    return guarded([&] {
        DeviceGuard g(ctx->device);
        const int b = yg::br_ctas_per_sm(ctx->logN, ctx->p.torus_bits, ctx->p.n, ctx->p.l_approx, per_cta, layout);
        if (b == yg::kNoVariant) {
            *out = 0;  // no kernel of that shape for these parameters: nothing fits
            return YG_OK;
        }
        if (b < 0) ck(cudaGetLastError(), "occupancy query");
        *out = b;
        return YG_OK;
    });
}

int yg_wait_timeouts(yg_ctx* ctx, uint64_t* out) {
    if (!ctx || !out) return set_err(YG_ERR_INVALID, "null argument");
    return guarded([&] {
        DeviceGuard g(ctx->device);
        unsigned long long v = 0;
        if (yg::read_wait_timeouts(&v) != 0) ck(cudaGetLastError(), "reading the wait-timeout counter");
        *out = v;
        return YG_OK;
    });
}

int yg_ctx_set_launch(yg_ctx* ctx, int layout, int per_cta, int ctas_per_sm) {
    if (!ctx || per_cta < 1 || ctas_per_sm < 0) return set_err(YG_ERR_INVALID, "yg_ctx_set_launch: bad arguments");
    int fit = 0;
    if (int rc = yg_ctas_per_sm(ctx, layout, per_cta, &fit)) return rc;
    if (fit < 1) return set_err(YG_ERR_INVALID, "yg_ctx_set_launch: a CTA of that shape does not fit an SM");
    ctx->layout = layout;
    ctx->per_cta = per_cta;
    ctx->ctas_per_sm = ctas_per_sm;
    ctx->launch_set = true;
    return YG_OK;
}

}  // extern "C"
