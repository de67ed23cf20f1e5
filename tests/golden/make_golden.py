"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Runs only where the reference tree is present: it builds oracle/_ref (the reference's
sources compiled against the HEXL/GMP stand-ins and the seeded RNG) and records, per
parameter set and key seed:
  * SHA-256 digests of the key material the reference generates from the seed
    (LWE key, RLWE key, NTT-domain BSK words, KSK words) -- small, but enough for any
    machine to confirm that the restatement regenerates the same keys;
  * input ciphertexts (symEncTlwe on the same RNG stream, right after key generation),
    the test polynomial, the reference's outputs of functionalBootstrappingMPNtt, its
    decryptions, and the blind-rotation accumulator of ciphertext 0 after a few CMux steps.

and, for the approximate-CRT blind rotation (blindRotateApproxCRTNtt on the torus Q_CRT), the
reference's residue key rows (small n: they are stored whole), an encrypted plaintext, the
rotation amounts, the rotated sample, its residue samples and its decryption.

    python tests/golden/make_golden.py [ginx] [wwl24] [lazy] [group] [crt]
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle.oracle import CrtReference, Reference  # noqa: E402
from yatfhe_gb300 import lut as lutmod  # noqa: E402
from yatfhe_gb300.params import T32_N1024, T56_N2048, WWL24_T32_N2048, WWL24_T56_N2048, small  # noqa: E402

CASES = {
    # name: (params, key seed, number of ciphertexts, message seed)
    "t32_n1024_seed5eed0001": (T32_N1024, 0x5EED0001, 8, 11),
    "t56_n2048_seed5eed0003": (T56_N2048, 0x5EED0003, 6, 12),
    "t32_n1024_small40_seed7": (small(T32_N1024, 40), 7, 16, 13),
}

WWL24_CASES = {
    # name: (params, key seed, number of ciphertexts, message seed); sign bootstrap
    "wwl24_t32_n2048_seed5eed0005": (WWL24_T32_N2048, 0x5EED0005, 8, 14),
    "wwl24_t56_n2048_seed5eed0006": (WWL24_T56_N2048, 0x5EED0006, 8, 15),
}

LAZY_CASES = {
    # name: (params, key seed, number of ciphertexts, message seed); sign bootstrap through
    # blindRotateLazyPipeAltNtt on the reference's default sets.  (On the n=630, N=1024 set
    # the reference's own lazy outputs do not decrypt: its s2 key has 3 levels of 7 bits.)
    "lazy_t32_n2048_seed5eed0007": (WWL24_T32_N2048, 0x5EED0007, 8, 16),
    "lazy_t56_n2048_seed5eed0008": (WWL24_T56_N2048, 0x5EED0008, 8, 17),
}

GROUP_CASES = {
    # name: (params, group, key seed, number of ciphertexts, message seed); sign bootstrap
    # through functionalBootstrappingNtt / blindRotateNtt with the group-g key family
    "group2_t32_n1024_seed5eed000c": (T32_N1024, 2, 0x5EED000C, 8, 19),
    "group3_t32_n1024_seed5eed000d": (T32_N1024, 3, 0x5EED000D, 8, 20),
    "group1_t32_n1024_seed5eed000e": (T32_N1024, 1, 0x5EED000E, 8, 21),
    "group2_t56_n2048_seed5eed000f": (T56_N2048, 2, 0x5EED000F, 8, 22),
}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def messages(p, count, seed):
    rng = np.random.default_rng(seed)
    if p.torus_bits == 32:
        bits = rng.integers(0, 2, count)
        mu = np.where(bits == 1, 1 << 29, -(1 << 29)).astype(np.int64)
        return mu, lutmod.sign_lut(p.N, 32), 8, np.where(bits == 1, 1, -1)
    m = rng.integers(0, 16, count)
    table = rng.integers(0, 16, 16)
    mu = (m * (1 << 27)).astype(np.int64)
    return mu, lutmod.padded_message_lut(p.N, 56, table), 32, table[m]


def make(name, p, seed, count, mseed):
    ref = Reference(p)
    ref.keygen(seed)
    s, z = ref.keys()
    bsk = ref.bsk_ntt()
    ksk = ref.ksk()
    mu, lut, base, expect = messages(p, count, mseed)
    lwe = ref.encrypt(mu)
    out = ref.pbs(lwe, lut, threads=1)
    dec = ref.decrypt(out, base)
    if not np.array_equal(dec, expect):
        raise SystemExit(f"{name}: the reference's own decryptions {dec} differ from the messages {expect}")
    cps = sorted({0, 1, p.n // 2, p.n - 1})
    acc, final = ref.blind_rotate_trace(lwe[0], lut, cps)
    np.savez_compressed(
        HERE / f"{name}.npz",
        params=np.array([p.n, p.N, p.k, p.radix_bits, p.l, p.l_approx, p.ks_radix_bits, p.ks_level, p.lwe_noise_b,
                         p.rlwe_noise_b, p.torus_base, p.torus_bits], np.int64),
        seed=np.array([seed], np.uint64),
        sha_lwe_s=digest(s), sha_rlwe_s=digest(z), sha_bsk=digest(bsk), sha_ksk=digest(ksk),
        mu=mu, lwe_in=lwe, lut=lut, lwe_out=out, decrypted=dec, base=np.array([base]),
        checkpoints=np.array(cps, np.int64), acc=acc, acc_final=final)
    print(f"{name}: {count} ciphertexts, outputs decrypt to the messages")


def make_wwl24(name, p, seed, count, mseed):
    ref = Reference(p)
    ref.keygen_wwl24(seed)
    s, z = ref.keys()
    cprime, s2 = ref.wwl24_words()
    expanded = ref.wwl24_expanded()
    ksk = ref.ksk()
    rng = np.random.default_rng(mseed)
    bits = rng.integers(0, 2, count)
    mu = np.where(bits == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lut = lutmod.sign_lut(p.N, p.torus_bits)
    lwe = ref.encrypt(mu)
    out, acc0 = ref.pbs_wwl24(lwe, lut, with_acc=True)
    dec = ref.decrypt(out, 8)
    expect = np.where(bits == 1, 1, -1)
    if not np.array_equal(dec, expect):
        raise SystemExit(f"{name}: the reference's own decryptions {dec} differ from the messages {expect}")
    np.savez_compressed(
        HERE / f"{name}.npz",
        params=np.array([p.n, p.N, p.k, p.radix_bits, p.l, p.l_approx, p.ks_radix_bits, p.ks_level, p.lwe_noise_b,
                         p.rlwe_noise_b, p.torus_base, p.torus_bits], np.int64),
        seed=np.array([seed], np.uint64),
        sha_lwe_s=digest(s), sha_rlwe_s=digest(z), sha_cprime=digest(cprime), sha_s2=digest(s2),
        sha_expanded=digest(expanded), sha_ksk=digest(ksk),
        mu=mu, lwe_in=lwe, lut=lut, lwe_out=out, decrypted=dec, base=np.array([8]), acc0=acc0)
    print(f"{name}: {count} ciphertexts, outputs decrypt to the messages")


def make_lazy(name, p, seed, count, mseed):
    ref = Reference(p)
    ref.keygen_lazy(seed)
    s, z = ref.keys()
    cprime, s2 = ref.lazy_words()
    ksk = ref.ksk()
    rng = np.random.default_rng(mseed)
    bits = rng.integers(0, 2, count)
    mu = np.where(bits == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lut = lutmod.sign_lut(p.N, p.torus_bits)
    lwe = ref.encrypt(mu)
    out, acc0 = ref.pbs_lazy(lwe, lut, with_acc=True)
    dec = ref.decrypt(out, 8)
    expect = np.where(bits == 1, 1, -1)
    if not np.array_equal(dec, expect):
        raise SystemExit(f"{name}: the reference's own decryptions {dec} differ from the messages {expect}")
    np.savez_compressed(
        HERE / f"{name}.npz",
        params=np.array([p.n, p.N, p.k, p.radix_bits, p.l, p.l_approx, p.ks_radix_bits, p.ks_level, p.lwe_noise_b,
                         p.rlwe_noise_b, p.torus_base, p.torus_bits], np.int64),
        seed=np.array([seed], np.uint64),
        sha_lwe_s=digest(s), sha_rlwe_s=digest(z), sha_cprime=digest(cprime), sha_s2=digest(s2),
        sha_ksk=digest(ksk),
        mu=mu, lwe_in=lwe, lut=lut, lwe_out=out, decrypted=dec, base=np.array([8]), acc0=acc0)
    print(f"{name}: {count} ciphertexts, outputs decrypt to the messages")


def make_group(name, p, group, seed, count, mseed):
    ref = Reference(p)
    ref.keygen_group(seed, group)
    s, z = ref.keys()
    words = ref.group_words()
    ksk = ref.ksk()
    rng = np.random.default_rng(mseed)
    bits = rng.integers(0, 2, count)
    mu = np.where(bits == 1, 1 << 29, -(1 << 29)).astype(np.int64)
    lut = lutmod.sign_lut(p.N, p.torus_bits)
    lwe = ref.encrypt(mu)
    out, acc0 = ref.pbs_group(lwe, lut, with_acc=True)
    dec = ref.decrypt(out, 8)
    expect = np.where(bits == 1, 1, -1)
    if not np.array_equal(dec, expect):
        raise SystemExit(f"{name}: the reference's own decryptions {dec} differ from the messages {expect}")
    np.savez_compressed(
        HERE / f"{name}.npz",
        params=np.array([p.n, p.N, p.k, p.radix_bits, p.l, p.l_approx, p.ks_radix_bits, p.ks_level, p.lwe_noise_b,
                         p.rlwe_noise_b, p.torus_base, p.torus_bits], np.int64),
        group=np.array([group]), seed=np.array([seed], np.uint64),
        sha_lwe_s=digest(s), sha_rlwe_s=digest(z), sha_key=digest(words), sha_ksk=digest(ksk),
        mu=mu, lwe_in=lwe, lut=lut, lwe_out=out, decrypted=dec, base=np.array([8]), acc0=acc0)
    print(f"{name}: {count} ciphertexts, outputs decrypt to the messages")


CRT_CASES = {
    # name: (n, N, key seed, message seed)
    "crt_n3_n2048_seed5eed0011": (3, 2048, 0x5EED0011, 21),
}


def make_crt(name, n, N, seed, mseed):
    r = CrtReference(n, N)
    r.keygen(seed)
    rng = np.random.default_rng(mseed)
    plain = rng.integers(-r.base // 2, r.base // 2, N).astype(np.int32)
    ct = r.encrypt(plain)
    rot = rng.integers(1, 2 * N, n).astype(np.int32)
    out, mcrt = r.blind_rotate(ct, rot)
    s = r.lwe_key()
    np.savez_compressed(HERE / f"{name}.npz", bsk8=r.bsk8(), acc_in=ct.astype(np.int32), rot=rot,
                        acc_out=out.astype(np.int32), mcrt=mcrt, plain=plain, lwe_s=s, dec=r.decrypt(out),
                        shift=np.array([int((rot.astype(np.int64) * s).sum()) % (2 * N)]))
    print(name)


if __name__ == "__main__":
    # optional arguments: the families to (re)generate, of "ginx", "wwl24", "lazy", "group", "crt"
    # (default all)
    families = set(sys.argv[1:]) or {"ginx", "wwl24", "lazy", "group", "crt"}
    if "ginx" in families:
        for name, (p, seed, count, mseed) in CASES.items():
            make(name, p, seed, count, mseed)
    if "wwl24" in families:
        for name, (p, seed, count, mseed) in WWL24_CASES.items():
            make_wwl24(name, p, seed, count, mseed)
    if "lazy" in families:
        for name, (p, seed, count, mseed) in LAZY_CASES.items():
            make_lazy(name, p, seed, count, mseed)
    if "group" in families:
        for name, (p, group, seed, count, mseed) in GROUP_CASES.items():
            make_group(name, p, group, seed, count, mseed)
    if "crt" in families:
        for name, (n, N, seed, mseed) in CRT_CASES.items():
            make_crt(name, n, N, seed, mseed)
