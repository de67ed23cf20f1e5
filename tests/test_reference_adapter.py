"""The C++ adapter header (include/yatfhe_gb300_reference.hpp) compiles against the
reference's own headers, i.e. a reference user can call the GPU path with the reference's
types and signatures.  Compile-only here (no GPU); needs the reference tree."""
import shutil
import subprocess
from pathlib import Path

import pytest

from oracle import oracle as o

ROOT = Path(__file__).resolve().parents[1]
REF_INC = o.REF_TREE / "yatfhe" / "include"

SRC = r"""
#include "yatfhe/bootstrapping.h"
#include "yatfhe/blind_rotate.h"
#include "yatfhe/keyswitching.h"
#include "yatfhe_gb300_reference.hpp"

void use(Tlwe& out, const Tlwe& in, const BootstrappingKeyMP& bsk, const TlweKeySwitchingKey& ksk,
         const TorusPolynomial& v, const YatfheParameters& p, Trlwe& acc, const ScaledTlwe& s,
         std::vector<Tlwe>& outs, const std::vector<Tlwe>& ins, const BootstrappingKeyWWL24& wwl,
         const BootstrappingKeyMPLazyPipeAlt& lazy, const std::vector<NttPolynomial>& gdV,
         const BootstrappingKey& gbsk, BootstrappingKeyMPLazyPipeAlt& lazy2, std::vector<Trlwe8>& acc8,
         const BootstrappingKeyCRT& crt) {
    yatfhe_gb300::functionalBootstrappingMPNtt(out, in, bsk, ksk, v, p);
    yatfhe_gb300::functionalBootstrappingMPNttBatch(outs, ins, bsk, ksk, v, p);
    yatfhe_gb300::blindRotateMP21Ntt(acc, bsk.bskDft, s, p);
    yatfhe_gb300::blindRotateJP22Ntt(acc, bsk, s, p);
    yatfhe_gb300::blindRotateWWL24Ntt(acc, wwl, s, p);
    yatfhe_gb300::blindRotateLazyPipeAltNtt(acc, lazy, s, v, gdV, p);
    yatfhe_gb300::blindRotateLazyPipeAltNttSweep(acc, lazy, s, v, gdV, 2, 2, p);
    yatfhe_gb300::blindRotateLazyPipeAltInitNtt(acc, lazy2, s, v, "BSK_OURS.bin", gdV, p);
    yatfhe_gb300::blindRotateLazyPipeAltNoFirstNtt(acc, lazy, s, v, p);
    yatfhe_gb300::blindRotateNtt(acc, gbsk.bskDft, s, p);
    yatfhe_gb300::functionalBootstrappingNtt(out, in, gbsk, ksk, v, p);
    yatfhe_gb300::switchKeyForTlwe(out, ksk, in, p);
    yatfhe_gb300::blindRotateApproxCRTNtt(acc8, crt.bskCRT, s, p);
    yatfhe_gb300::forgetKeys();
}
"""


@pytest.mark.skipif(not REF_INC.exists(), reason="reference headers not present")
@pytest.mark.parametrize("torus", ["TORUS32", "TORUS56"])
def test_adapter_compiles_against_reference_headers(tmp_path, torus):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    f = tmp_path / "use.cpp"
    f.write_text(SRC)
    cmd = [cxx, "-std=c++17", "-fsyntax-only", f"-D{torus}", f"-I{REF_INC}", f"-I{ROOT / 'oracle' / 'shim'}",
           f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include", str(f)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(not REF_INC.exists(), reason="reference headers not present")
def test_adapter_runs_against_the_reference(tmp_path):
    """The adapter run end to end in the shape of the reference's BOOTSTRAPPING.MP21 test
    (google_tests/bootstrappping_test.cpp:83-131): tests/adapter/adapter_run.cpp calls
    yatfhe_gb300::functionalBootstrappingMPNtt (single and batched), blindRotateMP21Ntt,
    blindRotateJP22Ntt, switchKeyForTlwe, the lazy rotations (blindRotateLazyPipeAltNtt and its
    Sweep, NoFirst and Init forms, the last reading a key file twice) and blindRotateApproxCRTNtt
    with the reference's own types and compares each
    result with the reference function itself on the same objects.  Below the adapter, the
    C ABI is a CPU stand-in built on the reference's functions (tests/adapter/yg_on_reference.cpp),
    so any error in the adapter's conversions changes a result; the GPU side of that ABI is
    covered by the -m gpu tests.  Also checked: the key cache converts a key once, a new key
    built at a freed key's address is recognised and uploaded again, and forgetKeys()."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    o.build_reference()
    lib_dir = ROOT / "oracle" / "_ref"
    exe = tmp_path / "adapter_run"
    src = ROOT / "tests" / "adapter"
    cmd = [cxx, "-std=c++17", "-O2", "-DNDEBUG", "-pthread", "-DUSING_NTT=HEXL", "-DTORUS32", f"-I{REF_INC}",
           f"-I{ROOT / 'oracle' / 'shim'}", f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include",
           str(src / "adapter_run.cpp"), str(src / "yg_on_reference.cpp"), f"-L{lib_dir}", "-lyatfhe_ref_t32",
           f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600, cwd=tmp_path,
                         env={**__import__("os").environ, "YATFHE_THREADS": "4"})
    assert run.returncode == 0, run.stdout + run.stderr
    assert "0 failure(s)" in run.stdout
