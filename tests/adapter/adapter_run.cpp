// adapter_run.cpp -- TEST INFRASTRUCTURE ONLY.  Runs the C++ adapter
// (include/yatfhe_gb300_reference.hpp) the way a reference user would, in the shape of the
// reference's own BOOTSTRAPPING.MP21 test (google_tests/bootstrappping_test.cpp:83-131), and
// compares every result with the reference function it replaces, called directly on the same
// objects.  Linked with the reference library built from its sources (oracle/_ref) and the
// CPU stand-in of the C ABI (yg_on_reference.cpp).  Exit status 0 when everything matches.
#include <cstdio>
#include <string>
#include <memory>
#include <new>
#include <vector>

#include "yatfhe/blind_rotate.h"
#include "yatfhe/bootstrapping.h"
#include "yatfhe/keyswitching.h"
#include "yatfhe/numeric.h"
#include "yatfhe/polynomial.h"
#include "yatfhe/tlwe.h"
#include "yatfhe/trlwe.h"
#include "yatfhe/trgsw.h"
#include "yautil/initializer.h"
#include "yautil/ya_serializer.h"
#include "yatfhe_gb300_reference.hpp"

extern "C" void yg_test_use_params(const YatfheParameters* p);
extern "C" int yg_test_uploads(void);
extern "C" int yg_test_crt_uploads(void);

namespace {

int failures = 0;

bool same(const Tlwe& x, const Tlwe& y) { return x.a == y.a && x.b == y.b; }
bool same(const Trlwe& x, const Trlwe& y) {
    for (size_t r = 0; r < x.a.size(); r++)
        if (x.a[r].coeffs != y.a[r].coeffs) return false;
    return x.b.coeffs == y.b.coeffs;
}

void expect(bool ok, const char* what) {
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    failures += !ok;
}

}  // namespace

int main() {
    YatfheParameters param{};
    param.n = 48;
    param.torusBase = 8;
    param.setRadixBits(7);
    param.l = 3;
    param.lApprox = 3;
    initYatfhe(param);
    yg_test_use_params(&param);

    TlweKey tlweKey{param.n};
    TrgswKey trgswKey{param};
    TrlweKey& trlweKey = trgswKey.trlweKey;
    TlweKeySwitchingKey ksKey{param};
    genTlweKey(tlweKey);
    genTrlweKey(trlweKey);
    // the bootstrapping key lives in storage the test can reuse for a second key
    alignas(BootstrappingKeyMP) unsigned char storage[sizeof(BootstrappingKeyMP)];
    auto* bsk = new (storage) BootstrappingKeyMP{param, param.lApprox};
    genBootstrappingKeyMP(*bsk, trgswKey, tlweKey, param);
    TlweKey tlweKsKey = tlweKey;
    genTlweKeySwitchingKey(ksKey, trlweKey, tlweKsKey, param);

    TorusPolynomial v{param.N};
    generateTestPolynomial(v, param.torusBase, 2 * param.N);
    std::vector<Tlwe> inputs;
    // messages in [0, torusBase / 2): the half the negacyclic test polynomial maps to itself
    // (the reference's test bootstraps 3 with torusBase 8)
    for (Integer m : {0, 1, 2, 3, 1, 3}) {
        Tlwe in{param.n};
        symEncTlwe(in, modSwitchToTorusGeneral(m, param.torusBase, LWE_Q), tlweKey);
        inputs.push_back(in);
    }

    // functionalBootstrappingMPNtt, one ciphertext at a time and batched
    bool pbs_ok = true, dec_ok = true;
    std::vector<Tlwe> want;
    for (const Tlwe& in : inputs) {
        Tlwe ref{param.n}, got{param.n};
        functionalBootstrappingMPNtt(ref, in, *bsk, ksKey, v, param);
        yatfhe_gb300::functionalBootstrappingMPNtt(got, in, *bsk, ksKey, v, param);
        pbs_ok &= same(ref, got);
        Tlwe in_copy = in;
        dec_ok &= symDecTlweToInt(got, tlweKey, param.torusBase) == symDecTlweToInt(in_copy, tlweKey, param.torusBase);
        want.push_back(ref);
    }
    expect(pbs_ok, "functionalBootstrappingMPNtt == the reference's");
    expect(dec_ok, "outputs decrypt to the inputs' messages");
    std::vector<Tlwe> outs;
    yatfhe_gb300::functionalBootstrappingMPNttBatch(outs, inputs, *bsk, ksKey, v, param);
    bool batch_ok = outs.size() == inputs.size();
    for (size_t i = 0; batch_ok && i < outs.size(); i++) batch_ok = same(outs[i], want[i]);
    expect(batch_ok, "functionalBootstrappingMPNttBatch == the reference's, per ciphertext");
    expect(yg_test_uploads() == 1, "the key was converted once and then taken from the cache");

    // blindRotateMP21Ntt / blindRotateJP22Ntt on a caller-built accumulator, then extraction
    // and switchKeyForTlwe
    ScaledTlwe scaled{param.N * 2, param.n};
    rescaleTlweToNewMod(scaled, inputs[3]);
    Trlwe acc_ref{param.k, param.N}, acc_got{param.k, param.N}, acc_jp{param.k, param.N};
    genNoiselessTrlweSample(acc_ref, v, scaled);
    acc_got = acc_ref;
    acc_jp = acc_ref;
    blindRotateMP21Ntt(acc_ref, bsk->bskDft, scaled, param);
    yatfhe_gb300::blindRotateMP21Ntt(acc_got, bsk->bskDft, scaled, param);
    yatfhe_gb300::blindRotateJP22Ntt(acc_jp, *bsk, scaled, param);
    expect(same(acc_ref, acc_got), "blindRotateMP21Ntt == the reference's");
    expect(same(acc_ref, acc_jp), "blindRotateJP22Ntt == blindRotateMP21Ntt of the reference");
    Tlwe big{ksKey.nCurrKey}, ks_ref{param.n}, ks_got{param.n};
    extractTlweFromTrlwe(big, acc_ref, param.driftPhase);
    switchKeyForTlwe(ks_ref, ksKey, big, param);
    yatfhe_gb300::switchKeyForTlwe(ks_got, ksKey, big, param);
    expect(same(ks_ref, ks_got), "switchKeyForTlwe == the reference's");
    expect(same(ks_ref, want[3]), "rotate + extract + switch == functionalBootstrappingMPNtt");

    // a new key built at the address of the old one: the cache must not serve the old one
    const int uploads = yg_test_uploads();
    bsk->~BootstrappingKeyMP();
    bsk = new (storage) BootstrappingKeyMP{param, param.lApprox};
    genBootstrappingKeyMP(*bsk, trgswKey, tlweKey, param);
    bool new_ok = true;
    for (const Tlwe& in : inputs) {
        Tlwe ref{param.n}, got{param.n};
        functionalBootstrappingMPNtt(ref, in, *bsk, ksKey, v, param);
        yatfhe_gb300::functionalBootstrappingMPNtt(got, in, *bsk, ksKey, v, param);
        new_ok &= same(ref, got);
    }
    expect(new_ok, "a new key at the same address gives the reference's results with the new key");
    expect(yg_test_uploads() == uploads + 1, "the new key was uploaded once");

    // forgetKeys() drops the cache: the next call converts the key again
    yatfhe_gb300::forgetKeys();
    Tlwe got{param.n}, ref{param.n};
    yatfhe_gb300::functionalBootstrappingMPNtt(got, inputs[0], *bsk, ksKey, v, param);
    functionalBootstrappingMPNtt(ref, inputs[0], *bsk, ksKey, v, param);
    expect(same(ref, got) && yg_test_uploads() == uploads + 2, "after forgetKeys() the key is converted again");

    yatfhe_gb300::forgetKeys();
    bsk->~BootstrappingKeyMP();

    // the lazy ("OURS") rotations on the reference's default T32 set with a small n: the adapter's
    // blindRotateLazyPipeAltNtt, its Sweep, NoFirst and Init (file) forms against the reference's
    {
        YatfheParameters lp{};
        lp.n = 16;
        initYatfhe(lp);
        yg_test_use_params(&lp);
        TlweKey lk{lp.n};
        TrgswKey tk{lp};
        genTlweKey(lk);
        genTrlweKey(tk.trlweKey);
        BootstrappingKeyMPLazyPipeAlt lazy{lp, lp.lApprox, true};
        for (int i = 0; i < lazy.n; i++) encryptTrgswMP(lazy.bskPrime[i], lk.s[i], tk, 0, lp);
        symEncTrlevWithKeyNtt(lazy.s2Dft, tk.trlweKey, tk.trlweKey.s, true, lp);
        TorusPolynomial lv{lp.N};
        for (int j = 0; j < lp.N; j++) lv.coeffs[j] = static_cast<Torus>((j % 4) - 2) << 29;
        Tlwe x{lp.n};
        symEncTlwe(x, static_cast<Torus>(1) << 30, lk);
        ScaledTlwe sc{2 * lp.N, lp.n};
        rescaleTlweToNewMod(sc, x);
        sc.a[2] = 0;  // a skipped step
        std::vector<NttPolynomial> gdV;
        prepareGdV(gdV, lv, lp);
        Trlwe want{lp.k, lp.N}, got{lp.k, lp.N};
        ::blindRotateLazyPipeAltNtt(want, lazy, sc, lv, gdV, lp);
        const int up0 = yg_test_uploads();
        yatfhe_gb300::blindRotateLazyPipeAltNtt(got, lazy, sc, lv, gdV, lp);
        expect(same(want, got), "blindRotateLazyPipeAltNtt equals the reference's");
        Trlwe sweep{lp.k, lp.N};
        yatfhe_gb300::blindRotateLazyPipeAltNttSweep(sweep, lazy, sc, lv, gdV, 3, 1, lp);
        expect(same(want, sweep) && yg_test_uploads() == up0 + 1, "Sweep form: same result, key converted once");
        Trlwe nf{lp.k, lp.N}, nfRef{lp.k, lp.N};
        ::blindRotateLazyPipeAltNoFirstNtt(nfRef, lazy, sc, lv, lp);
        yatfhe_gb300::blindRotateLazyPipeAltNoFirstNtt(nf, lazy, sc, lv, lp);
        expect(same(nfRef, nf), "blindRotateLazyPipeAltNoFirstNtt equals the reference's");
        const std::string file = "adapter_run_lazy_key.bin";
        serializeBskLazyPipeAlt(lazy, file);
        BootstrappingKeyMPLazyPipeAlt holder{lp, lp.lApprox, true};
        Trlwe init1{lp.k, lp.N}, init2{lp.k, lp.N};
        const int up1 = yg_test_uploads();
        yatfhe_gb300::blindRotateLazyPipeAltInitNtt(init1, holder, sc, lv, file, gdV, lp);
        yatfhe_gb300::blindRotateLazyPipeAltInitNtt(init2, holder, sc, lv, file, gdV, lp);
        expect(same(want, init1) && same(want, init2) && yg_test_uploads() == up1 + 2,
               "InitNtt form: the key read from the file, uploaded again on each call");
        bool refused = false;
        try {
            yatfhe_gb300::blindRotateLazyPipeAltNttSweep(sweep, lazy, sc, lv, gdV, 0, 1, lp);
        } catch (const std::invalid_argument&) {
            refused = true;
        }
        expect(refused, "Sweep form: moveNtt < 1 refused");
        std::remove(file.c_str());
        yatfhe_gb300::forgetKeys();
    }

    // blindRotateApproxCRTNtt in the setting of the reference's BLIND_ROT_APPROX_CRT_NTT test
    // (google_tests/blindrot_test.cpp:574-640): the torus Q_CRT, its own key generation and
    // encryption; param.l = dh keeps encryptTrgswApproxCRT inside its gadget vector
    {
        YatfheParameters cp{};
        cp.q = Q_CRT;
        cp.n = 12;
        cp.l = cp.dh;
        initYatfhe(cp);
        yg_test_use_params(&cp);
        TlweKey lk{cp.n};
        TrgswKey tk{cp};
        genTlweKey(lk);
        genTrlweKey(tk.trlweKey);
        BootstrappingKeyCRT crtKey{cp};
        genBootstrappingKeyApproxCrt(crtKey, tk, lk, cp);
        std::vector<Torus> mu(cp.N);
        for (int j = 0; j < cp.N; j++) mu[j] = modSwitchToTorus32(j % cp.torusBase - cp.torusBase / 2, cp.torusBase);
        Trlwe in{cp.k, cp.N};
        symEncTrlweMultiSample(in, tk.trlweKey, mu);
        ScaledTlwe s{2 * cp.N, cp.n};
        for (int i = 0; i < cp.n; i++) s.a[i] = (i * 577 + 13) % (4 * cp.N) - 2 * cp.N;
        s.a[3] = 0;
        std::vector<Trlwe8> want(cp.d, Trlwe8{cp.k, cp.N});
        decompTrlweMcrt(want, in, cp);
        std::vector<Trlwe8> got = want;
        ::blindRotateApproxCRTNtt(want, crtKey.bskCRT, s, cp);
        const int before = yg_test_crt_uploads();
        yatfhe_gb300::blindRotateApproxCRTNtt(got, crtKey.bskCRT, s, cp);
        auto same8 = [&](const std::vector<Trlwe8>& x, const std::vector<Trlwe8>& y) {
            for (int d = 0; d < cp.d; d++)
                if (x[d].a[0].coeffs != y[d].a[0].coeffs || x[d].b.coeffs != y[d].b.coeffs) return false;
            return true;
        };
        expect(same8(want, got), "blindRotateApproxCRTNtt equals the reference's");
        std::vector<Trlwe8> again(cp.d, Trlwe8{cp.k, cp.N});
        decompTrlweMcrt(again, in, cp);
        yatfhe_gb300::blindRotateApproxCRTNtt(again, crtKey.bskCRT, s, cp);
        expect(same8(want, again) && yg_test_crt_uploads() == before + 1,
               "blindRotateApproxCRTNtt converts its key once");
        yatfhe_gb300::forgetKeys();
    }
    std::printf("%d failure(s)\n", failures);
    return failures ? 1 : 0;
}
