"""Parameter sets of the bootstrap path.

Mirrors the fields of the reference's ``YatfheParameters`` that the GINX/MP21 bootstrap
reads (yatfhe/include/yatfhe/yatfhe_parameters.h:9-110): LWE dimension ``n``, ring degree
``N``, ``k``, gadget radix bits and levels, key-switching radix bits and levels, the
TUniform noise exponents and the torus width.  ``l_approx`` is the number of gadget
levels a key is generated with and decomposed into (``BootstrappingKeyMP(p, p.lApprox)``,
google_tests/bootstrappping_test.cpp:92).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, fields

# NTT primes of the two torus builds (yatfhe/include/yatfhe/torus.h:151,157).
Q_NTT = {32: 562941363486721, 56: 1945555039024054273}


@dataclass(frozen=True)
class PbsParams:
    n: int
    N: int
    k: int
    radix_bits: int
    l: int
    l_approx: int
    ks_radix_bits: int
    ks_level: int
    lwe_noise_b: int
    rlwe_noise_b: int
    torus_base: int
    torus_bits: int

    @property
    def q_ntt(self) -> int:
        return Q_NTT[self.torus_bits]

    @property
    def lwe_words(self) -> int:
        """int32 words of one LWE ciphertext [a_0..a_{n-1}, b]."""
        return self.n + 1

    @property
    def bsk_ntt_words(self) -> int:
        """uint64 words of the NTT-domain bootstrapping key, [n][l][k+1][k+1][N]."""
        return self.n * self.l_approx * (self.k + 1) ** 2 * self.N

    @property
    def ksk_words(self) -> int:
        """int32 words of the key-switching key, [k N][t][n+1]."""
        return self.k * self.N * self.ks_level * (self.n + 1)

    def bsk_file_bytes(self) -> int:
        """Size of the reference's BSK file for these parameters (ya_serializer.cpp:276-285)."""
        k, N, L = self.k, self.N, self.l_approx
        trlwe_dft = 4 + 1 + (4 + 8 * N) + 4 + k * (4 + 8 * N)
        trgsw = 4 + 4 + 1 + 4 + L * (4 + k * trlwe_dft) + 4 + L * trlwe_dft
        return self.n * trgsw + 4 + 4 + 1

    def validate(self) -> None:
        if self.torus_bits not in (32, 56):
            raise ValueError("torus_bits must be 32 or 56")
        if self.N & (self.N - 1) or not 256 <= self.N <= 2048:
            raise ValueError("N must be a power of two in [256, 2048]")
        if self.k != 1:
            raise ValueError("only k = 1 is supported")
        if self.l_approx * self.radix_bits > self.torus_bits:
            raise ValueError("l * radixBits exceeds the torus width")
        if self.ks_level * self.ks_radix_bits > 32:
            raise ValueError("ksLevel * ksRadixBits exceeds the 32-bit LWE modulus")

    def as_ctypes(self):
        return _CParams(*(getattr(self, f.name) for f in fields(self)))


class _CParams(ctypes.Structure):
    _fields_ = [(f.name, ctypes.c_int) for f in fields(PbsParams)]


# TORUS=32 set: n=630, N=1024, B=2^7, l=3, KS 2^2 x 8, TUniform exponents 18 (LWE) and 8
# (RLWE, sigma = 2^-25 in torus units).
T32_N1024 = PbsParams(n=630, N=1024, k=1, radix_bits=7, l=3, l_approx=3, ks_radix_bits=2, ks_level=8,
                      lwe_noise_b=18, rlwe_noise_b=8, torus_base=8, torus_bits=32)

# TORUS=56 set: n=750, N=2048, B=2^10, l=4, KS 2^3 x 10, RLWE exponent 17 (sigma = 2^-40).
# The LWE/KSK exponent is 14 (sigma ~ 2^-19), not 18 (sigma = 2^-15): with 2^-15 the
# 2048 x 10 key-switching terms alone leave a noise of about half a slot of a 4-bit padded
# message, and the reference's own outputs misdecrypt about a quarter of them.
T56_N2048 = PbsParams(n=750, N=2048, k=1, radix_bits=10, l=4, l_approx=4, ks_radix_bits=3, ks_level=10,
                      lwe_noise_b=14, rlwe_noise_b=17, torus_base=32, torus_bits=56)

# The reference's default parameter sets (yatfhe/include/yatfhe/yatfhe_parameters.h:9-40,
# setKsRadixBits(2) -> ksLevel 16), on which its WWL+24 test runs: blind rotation with
# lApprox levels, the s2 key of the WWL+24 family with l levels.
WWL24_T32_N2048 = PbsParams(n=680, N=2048, k=1, radix_bits=4, l=8, l_approx=4, ks_radix_bits=2, ks_level=16,
                            lwe_noise_b=18, rlwe_noise_b=3, torus_base=4, torus_bits=32)
WWL24_T56_N2048 = PbsParams(n=680, N=2048, k=1, radix_bits=14, l=4, l_approx=1, ks_radix_bits=2, ks_level=16,
                            lwe_noise_b=18, rlwe_noise_b=8, torus_base=4, torus_bits=56)

# Reduced-n variants of the two sets (same ring, gadget and key-switching parameters, fewer
# CMux steps); used where the oracle must finish in seconds.
def small(p: PbsParams, n: int) -> PbsParams:
    from dataclasses import replace

    return replace(p, n=n)


PARAM_SETS = {"t32_n1024": T32_N1024, "t56_n2048": T56_N2048}
