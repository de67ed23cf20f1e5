"""Test-polynomial (LUT) builders in the reference's box layouts.

``sign_lut`` is the constant polynomial of a sign bootstrap.  ``box_lut`` generalises
generateTestPolynomialFR (yatfhe/src/polynomial.cpp:92-107) to arbitrary slot values:
slot s (s = 0 .. p-1) covers N/p consecutive rotation amounts centred on s N/p, slot 0's
lower half wraps to the top of the array negated, exactly as the reference lays out
its full-range LUT.  With values[s] = intModP(s, p) 2^T / p it reproduces that function.
"""
from __future__ import annotations

import numpy as np


def _sext(x: np.ndarray, bits: int) -> np.ndarray:
    x = np.asarray(x, dtype=np.int64)
    sh = 64 - bits
    return ((x.astype(np.uint64) << np.uint64(sh)).astype(np.int64)) >> sh


def sign_lut(N: int, torus_bits: int, value: int | None = None) -> np.ndarray:
    """v = value everywhere (default 2^T / 8): bootstraps phase in [0, 1/2) to +value, else -value."""
    v = (1 << (torus_bits - 3)) if value is None else value
    return np.full(N, v, dtype=np.int64)


def box_lut(N: int, torus_bits: int, slot_values) -> np.ndarray:
    vals = np.asarray(slot_values, dtype=np.int64)
    p = len(vals)
    if N % p or (N // p) % 2:
        raise ValueError("N / p must be an even integer")
    width = N // p
    half = width // 2
    t = _sext(vals[np.arange(N) // width], torus_bits)
    t[:half] = _sext(-t[:half], torus_bits)
    return np.roll(t, -half)


def padded_message_lut(N: int, torus_bits: int, table, base: int = 32) -> np.ndarray:
    """LUT for messages m in [0, len(table)) encoded as m 2^32 / base (one padding bit when
    len(table) == base / 2): slot m returns table[m] 2^T / base."""
    table = np.asarray(table, dtype=np.int64)
    return box_lut(N, torus_bits, table * ((1 << torus_bits) // base))
