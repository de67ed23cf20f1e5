"""Python view of the C ABI, for tests, the benchmark and scripting.

Names follow the reference's C++ entry points (yatfhe/include/yatfhe/*.h) in snake case:

  Context                          initYatfhe + YatfheParameters (one parameter set)
  BootstrapKey.from_file           deserializeBskMP (yatfhe/src/ya_serializer.cpp:287-303)
  BootstrapKey.from_ntt_words      BootstrappingKeyMP::bskDft already in memory
  BootstrapKey.set_ksk             TlweKeySwitchingKey (yatfhe/include/yatfhe/keyswitching.h:14-31)
  functional_bootstrapping_mp_ntt  functionalBootstrappingMPNtt (yatfhe/src/bootstrapping.cpp:71-80)
  blind_rotate_mp21_ntt            rescaleTlweToNewMod + genNoiselessTrlweSample + blindRotateMP21Ntt
  switch_key_for_tlwe              switchKeyForTlwe (yatfhe/src/keyswitching.cpp:48-72)

Device arguments are torch CUDA tensors (int32 ciphertext words, int64 torus LUT words);
work is enqueued on torch's current stream.  ``*_host`` variants take numpy arrays.
Errors raise the Python counterpart of the reference's exceptions (ValueError for
std::invalid_argument, OSError for the serializer's std::runtime_error).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .params import PbsParams


def _torch():
    import torch

    return torch


def _stream_handle(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dptr(t, dtype_name: str, what: str):
    torch = _torch()
    want = getattr(torch, dtype_name)
    if not t.is_cuda or t.dtype != want or not t.is_contiguous():
        raise ValueError(f"{what} must be a contiguous CUDA tensor of {dtype_name}")
    return ctypes.c_void_p(t.data_ptr())


class Context:
    def __init__(self, params: PbsParams, device: int = 0):
        params.validate()
        self.params = params
        self.device = device
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_ctx_create(ctypes.byref(_lib.YgParams.of(params)), device, ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().yg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BootstrapKey:
    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self._h = handle
        # key format it was made from: "ginx" (BootstrappingKeyMP), "wwl24", "lazy" or
        # "group<g>" (BootstrappingKey with param.group = g)
        self.family = "ginx"

    @classmethod
    def from_file(cls, ctx: Context, path) -> "BootstrapKey":
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_key_load_bsk_file(ctx.handle, str(path).encode(), ctypes.byref(h)))
        return cls(ctx, h)

    @classmethod
    def from_ntt_words(cls, ctx: Context, words: np.ndarray) -> "BootstrapKey":
        w = np.ascontiguousarray(words, np.uint64)
        if w.size != ctx.params.bsk_ntt_words:
            raise ValueError(f"expected {ctx.params.bsk_ntt_words} NTT words, got {w.size}")
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_key_upload_bsk_ntt(ctx.handle, ctypes.c_void_p(w.ctypes.data), ctypes.byref(h)))
        return cls(ctx, h)

    @classmethod
    def from_wwl24_words(cls, ctx: Context, cprime: np.ndarray, s2: np.ndarray) -> "BootstrapKey":
        """A WWL+24 key (BootstrappingKeyWWL24: cPrime rows [n][l_approx][k+1][N] and the s2 key
        [levels][k+1][N], NTT-domain words mod q).  The GPU derives the GINX rows the WWL+24 blind
        rotation uses once, at upload; every entry point then gives the WWL+24 results."""
        p = ctx.params
        c = np.ascontiguousarray(cprime, np.uint64)
        s = np.ascontiguousarray(s2, np.uint64)
        row = (p.k + 1) * p.N
        if c.size != p.n * p.l_approx * row:
            raise ValueError(f"expected {p.n * p.l_approx * row} cPrime words, got {c.size}")
        if s.size == 0 or s.size % row:
            raise ValueError(f"the s2 key must be a whole number of [{p.k + 1}][{p.N}] levels")
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_key_upload_wwl24_ntt(ctx.handle, ctypes.c_void_p(c.ctypes.data),
                                                       ctypes.c_void_p(s.ctypes.data), s.size // row, ctypes.byref(h)))
        key = cls(ctx, h)
        key.family = "wwl24"
        return key

    @classmethod
    def from_wwl24_file(cls, ctx: Context, path) -> "BootstrapKey":
        """A WWL+24 key file written by serializeBskWWL24."""
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_key_load_wwl24_file(ctx.handle, str(path).encode(), ctypes.byref(h)))
        key = cls(ctx, h)
        key.family = "wwl24"
        return key

    @classmethod
    def from_lazy_words(cls, ctx: Context, cprime: np.ndarray, s2: np.ndarray) -> "BootstrapKey":
        """A lazy ("OURS") key (BootstrappingKeyMPLazyPipeAlt: half rows bskPrime[i].cPrime
        [n][l_approx][k+1][N] as torus values, the s2 key [levels][k+1][N] as NTT-domain words
        mod q).  The device keeps the rows in the torus word size; every bootstrap rebuilds each
        step's TRGSW from them (blindRotateLazyPipeAltNtt)."""
        p = ctx.params
        c = np.ascontiguousarray(cprime, np.int64)
        s = np.ascontiguousarray(s2, np.uint64)
        row = (p.k + 1) * p.N
        if c.size != p.n * p.l_approx * row:
            raise ValueError(f"expected {p.n * p.l_approx * row} half-row words, got {c.size}")
        if s.size == 0 or s.size % row:
            raise ValueError(f"the s2 key must be a whole number of [{p.k + 1}][{p.N}] levels")
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_key_upload_lazy(ctx.handle, ctypes.c_void_p(c.ctypes.data),
                                                  ctypes.c_void_p(s.ctypes.data), s.size // row, ctypes.byref(h)))
        key = cls(ctx, h)
        key.family = "lazy"
        return key

    @classmethod
    def from_lazy_file(cls, ctx: Context, path) -> "BootstrapKey":
        """A lazy key file written by serializeBskLazyPipeAlt."""
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_key_load_lazy_file(ctx.handle, str(path).encode(), ctypes.byref(h)))
        key = cls(ctx, h)
        key.family = "lazy"
        return key

    @classmethod
    def from_group_words(cls, ctx: Context, words: np.ndarray, group: int) -> "BootstrapKey":
        """A group-g key of blindRotateNtt (BootstrappingKey: TrgswDft words [keys][l][k+1][k+1][N],
        NTT domain mod q; keys = n for group 1, n / g * 2^g otherwise)."""
        p = ctx.params
        w = np.ascontiguousarray(words, np.uint64)
        keys = p.n if group == 1 else (p.n // group) << group
        per = (p.k + 1) ** 2 * p.N
        if w.size % (keys * per):
            raise ValueError(f"expected {keys} keys of [l][{p.k + 1}][{p.k + 1}][{p.N}] words")
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_key_upload_group(ctx.handle, ctypes.c_void_p(w.ctypes.data), group,
                                                  w.size // (keys * per), ctypes.byref(h)))
        key = cls(ctx, h)
        key.family = f"group{group}"
        return key

    def set_ksk(self, ksk: np.ndarray) -> "BootstrapKey":
        k = np.ascontiguousarray(ksk, np.int32)
        if k.size != self.ctx.params.ksk_words:
            raise ValueError(f"expected {self.ctx.params.ksk_words} KSK words, got {k.size}")
        _lib.check(_lib.lib().yg_key_set_ksk(self._h, ctypes.c_void_p(k.ctypes.data)))
        return self

    @property
    def handle(self):
        return self._h

    @property
    def device_bytes(self) -> int:
        return int(_lib.lib().yg_key_device_bytes(self._h))

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().yg_key_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchPlan:
    """A batch of `count` ciphertexts under several keys / LUTs (yg_plan_*): key_ids[c] and
    lut_ids[c] pick the key and LUT of ciphertext c.  run() only launches kernels, so it can be
    captured in a CUDA graph."""

    def __init__(self, ctx: Context, keys, luts, count: int, key_ids=None, lut_ids=None, grid: int = 0,
                 per_cta: int = 0, layout: int = 0):
        self.ctx, self.keys, self.luts, self.count = ctx, list(keys), list(luts), count
        kt = (ctypes.c_void_p * len(self.keys))(*[k.handle.value for k in self.keys])
        lt = (ctypes.c_void_p * len(self.luts))(*[ctypes.c_void_p(t.data_ptr()).value for t in self.luts])
        kid = None if key_ids is None else np.ascontiguousarray(key_ids, np.int32)
        lid = None if lut_ids is None else np.ascontiguousarray(lut_ids, np.int32)
        for ids in (kid, lid):
            if ids is not None and len(ids) != count:
                raise ValueError("index arrays must have one entry per ciphertext")
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_plan_create(
            ctx.handle, ctypes.cast(kt, ctypes.c_void_p), len(self.keys),
            None if kid is None else ctypes.c_void_p(kid.ctypes.data),
            ctypes.cast(lt, ctypes.c_void_p), len(self.luts),
            None if lid is None else ctypes.c_void_p(lid.ctypes.data), count, ctypes.byref(h)))
        self._h = h
        if grid or per_cta or layout:
            self.set_launch(per_cta or 1, grid, layout)

    def set_launch(self, per_cta: int, grid: int = 0, layout: int = 0):
        _lib.check(_lib.lib().yg_plan_set_launch(self._h, int(layout), int(per_cta), int(grid)))

    def run(self, lwe_in, out, stream=None):
        _lib.check(_lib.lib().yg_plan_run(self._h, _dptr(lwe_in, "int32", "lwe_in"), _dptr(out, "int32", "out"),
                                          _stream_handle(stream)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().yg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ctas_per_sm(ctx: Context, per_cta: int = 1, layout: int = 0) -> int:
    """CTAs of `per_cta` ciphertexts in `layout` (_lib.LAYOUT_*) that fit one SM (0: none)."""
    v = ctypes.c_int()
    _lib.check(_lib.lib().yg_ctas_per_sm(ctx.handle, int(layout), int(per_cta), ctypes.byref(v)))
    return v.value


def set_launch(ctx: Context, per_cta: int, ctas_per_sm: int = 0, layout: int = 0) -> None:
    _lib.check(_lib.lib().yg_ctx_set_launch(ctx.handle, int(layout), int(per_cta), int(ctas_per_sm)))


def functional_bootstrapping_mp_ntt(ctx: Context, key: BootstrapKey, lwe_in, lut, out=None, stream=None):
    """Bootstraps every row of ``lwe_in`` ([count, n+1] int32 CUDA tensor) through ``lut``."""
    torch = _torch()
    n1 = ctx.params.n + 1
    if lwe_in.dim() != 2 or lwe_in.shape[1] != n1:
        raise ValueError(f"lwe_in must have shape [count, {n1}]")
    if out is None:
        out = torch.empty_like(lwe_in)
    _lib.check(_lib.lib().yg_pbs(ctx.handle, key.handle, _dptr(lwe_in, "int32", "lwe_in"),
                                 _dptr(out, "int32", "out"), lwe_in.shape[0], _dptr(lut, "int64", "lut"),
                                 _stream_handle(stream)))
    return out


def functional_bootstrapping_mp_ntt_host(ctx: Context, key: BootstrapKey, lwe_in: np.ndarray, lut: np.ndarray,
                                         out: np.ndarray | None = None) -> np.ndarray:
    """Host-buffer form: copies in, bootstraps, copies out (pinned buffers give the fastest copies)."""
    a = np.ascontiguousarray(lwe_in, np.int32).reshape(-1, ctx.params.n + 1)
    v = np.ascontiguousarray(lut, np.int64)
    if out is None:
        out = np.empty_like(a)
    _lib.check(_lib.lib().yg_pbs_host(ctx.handle, key.handle, ctypes.c_void_p(a.ctypes.data),
                                      ctypes.c_void_p(out.ctypes.data), len(a), ctypes.c_void_p(v.ctypes.data),
                                      ctypes.c_void_p(0)))
    return out


def blind_rotate_mp21_ntt(ctx: Context, key: BootstrapKey, lwe_in, lut, steps: int | None = None, stream=None):
    """Accumulators [count, (k+1) N] (int64 torus words) after ``steps`` CMux steps (default n)."""
    torch = _torch()
    p = ctx.params
    steps = p.n if steps is None else steps
    acc = torch.empty((lwe_in.shape[0], (p.k + 1) * p.N), dtype=torch.int64, device=lwe_in.device)
    _lib.check(_lib.lib().yg_blind_rotate(ctx.handle, key.handle, _dptr(lwe_in, "int32", "lwe_in"),
                                          _dptr(lut, "int64", "lut"), _dptr(acc, "int64", "acc"),
                                          lwe_in.shape[0], steps, _stream_handle(stream)))
    return acc


def keygen_from_samples(ctx: Context, samples: dict, return_keys: bool = False):
    """Key generation on the GPU from caller-drawn random samples (yg_keygen_from_samples):
    `samples` holds lwe_s [n], rlwe_s [kN], bsk_noise [n][l][k+1][N], bsk_mask
    [n][l][k+1][k][N], ksk_mask [kN][t][n], ksk_noise [kN][t].  Returns the device key, and
    with return_keys also the NTT-domain BSK words and the KSK."""
    p = ctx.params
    k1, kN = p.k + 1, p.k * p.N
    shapes = {"lwe_s": (p.n,), "rlwe_s": (kN,), "bsk_noise": (p.n, p.l_approx, k1, p.N),
              "bsk_mask": (p.n, p.l_approx, k1, p.k, p.N), "ksk_mask": (kN, p.ks_level, p.n),
              "ksk_noise": (kN, p.ks_level)}
    arr = {}
    for name, shape in shapes.items():
        dt = np.uint64 if name == "bsk_mask" else np.int32
        x = np.ascontiguousarray(samples[name], dt)
        if x.size != int(np.prod(shape)):
            raise ValueError(f"{name}: expected {shape}, got {x.shape}")
        arr[name] = x
    words = np.zeros(p.bsk_ntt_words, np.uint64) if return_keys else None
    ksk = np.zeros(p.ksk_words, np.int32) if return_keys else None
    h = ctypes.c_void_p()
    ptr = lambda x: ctypes.c_void_p(x.ctypes.data) if x is not None else None  # noqa: E731
    _lib.check(_lib.lib().yg_keygen_from_samples(ctx.handle, ptr(arr["lwe_s"]), ptr(arr["rlwe_s"]),
                                                 ptr(arr["bsk_noise"]), ptr(arr["bsk_mask"]), ptr(arr["ksk_mask"]),
                                                 ptr(arr["ksk_noise"]), ptr(words), ptr(ksk), ctypes.byref(h)))
    key = BootstrapKey(ctx, h)
    return (key, words, ksk) if return_keys else key


def keygen(ctx: Context, seed: int, lwe_noise_b: int, rlwe_noise_b: int, return_secrets: bool = False):
    """Key generation with every random value drawn on the GPU (yg_keygen): ChaCha20 counter
    mode keyed by `seed`, the reference's distributions (binary secrets, TUniform noise,
    uniform masks).  Returns the device key (with BSK and KSK), and with return_secrets also
    the secrets (lwe_s [n], rlwe_s [kN] int32)."""
    p = ctx.params
    lwe_s = np.zeros(p.n, np.int32)
    rlwe_s = np.zeros(p.k * p.N, np.int32)
    h = ctypes.c_void_p()
    _lib.check(_lib.lib().yg_keygen(ctx.handle, seed, lwe_noise_b, rlwe_noise_b, ctypes.c_void_p(lwe_s.ctypes.data),
                                    ctypes.c_void_p(rlwe_s.ctypes.data), ctypes.byref(h)))
    key = BootstrapKey(ctx, h)
    return (key, lwe_s, rlwe_s) if return_secrets else key


def draw_keygen_samples(ctx: Context, seed: int, lwe_noise_b: int, rlwe_noise_b: int) -> dict:
    """The random samples keygen(seed) draws, in the layouts keygen_from_samples takes."""
    p = ctx.params
    k1, kN = p.k + 1, p.k * p.N
    d = {"lwe_s": np.zeros(p.n, np.int32), "rlwe_s": np.zeros(kN, np.int32),
         "bsk_noise": np.zeros((p.n, p.l_approx, k1, p.N), np.int32),
         "bsk_mask": np.zeros((p.n, p.l_approx, k1, p.k, p.N), np.uint64),
         "ksk_mask": np.zeros((kN, p.ks_level, p.n), np.int32),
         "ksk_noise": np.zeros((kN, p.ks_level), np.int32)}
    ptrs = [ctypes.c_void_p(d[f].ctypes.data) for f in ("lwe_s", "rlwe_s", "bsk_noise", "bsk_mask", "ksk_mask",
                                                         "ksk_noise")]
    _lib.check(_lib.lib().yg_draw_keygen_samples(ctx.handle, seed, lwe_noise_b, rlwe_noise_b, *ptrs))
    return d


def sym_enc_tlwe(ctx: Context, lwe_s, mu, seed: int, call: int, lwe_noise_b: int, out=None, stream=None):
    """symEncTlwe (yatfhe/src/tlwe.cpp:21-31) of the messages `mu` (int64 [count], torus mod
    2^32) under the binary secret `lwe_s` (int32 [n]), all on the GPU with masks and noise
    drawn from (seed, call): ciphertexts [count, n + 1] int32."""
    torch = _torch()
    n1 = ctx.params.n + 1
    if out is None:
        out = torch.empty((mu.shape[0], n1), dtype=torch.int32, device=mu.device)
    _lib.check(_lib.lib().yg_encrypt_lwe(ctx.handle, _dptr(lwe_s, "int32", "lwe_s"), _dptr(mu, "int64", "mu"),
                                         mu.shape[0], seed, call, lwe_noise_b, _dptr(out, "int32", "out"),
                                         _stream_handle(stream)))
    return out


def sym_enc_tlwe_from_samples(ctx: Context, lwe_s, mu, mask, noise, out=None, stream=None):
    """sym_enc_tlwe with the masks (int32 [count, n]) and noise (int32 [count]) given."""
    torch = _torch()
    n1 = ctx.params.n + 1
    if out is None:
        out = torch.empty((mu.shape[0], n1), dtype=torch.int32, device=mu.device)
    _lib.check(_lib.lib().yg_encrypt_lwe_from_samples(
        ctx.handle, _dptr(lwe_s, "int32", "lwe_s"), _dptr(mu, "int64", "mu"), _dptr(mask, "int32", "mask"),
        _dptr(noise, "int32", "noise"), mu.shape[0], _dptr(out, "int32", "out"), _stream_handle(stream)))
    return out


def _dptr_words(t, what: str):
    """A contiguous CUDA tensor of 64-bit words (uint64, or int64 holding the same bits)."""
    torch = _torch()
    if not t.is_cuda or t.dtype not in (torch.int64, getattr(torch, "uint64", torch.int64)) or not t.is_contiguous():
        raise ValueError(f"{what} must be a contiguous CUDA tensor of uint64 or int64")
    return ctypes.c_void_p(t.data_ptr())


def sym_enc_trlwe_ntt(ctx: Context, rlwe_s, mu, seed: int, call: int, rlwe_noise_b: int, out=None, stream=None):
    """symEncTrlweMultiSampleSimple (yatfhe/src/trlwe.cpp:40-47,62-64) of the torus polynomials
    `mu` (int64 [count, N]) under the binary secret `rlwe_s` (int32 [kN]), on the GPU with masks
    and noise drawn from (seed, call): NTT-domain samples [count, k+1, N] of words mod q
    (int64 tensor holding the uint64 words)."""
    torch = _torch()
    p = ctx.params
    if out is None:
        out = torch.empty((mu.shape[0], p.k + 1, p.N), dtype=torch.int64, device=mu.device)
    _lib.check(_lib.lib().yg_encrypt_rlwe_ntt(ctx.handle, _dptr(rlwe_s, "int32", "rlwe_s"), _dptr(mu, "int64", "mu"),
                                              mu.shape[0], seed, call, rlwe_noise_b, _dptr_words(out, "out"),
                                              _stream_handle(stream)))
    return out


def sym_enc_trlwe_ntt_from_samples(ctx: Context, rlwe_s, mu, mask, noise, out=None, stream=None):
    """sym_enc_trlwe_ntt with the masks (words [count, k, N]) and noise (int32 [count, N]) given."""
    torch = _torch()
    p = ctx.params
    if out is None:
        out = torch.empty((mu.shape[0], p.k + 1, p.N), dtype=torch.int64, device=mu.device)
    _lib.check(_lib.lib().yg_encrypt_rlwe_ntt_from_samples(
        ctx.handle, _dptr(rlwe_s, "int32", "rlwe_s"), _dptr(mu, "int64", "mu"), _dptr_words(mask, "mask"),
        _dptr(noise, "int32", "noise"), mu.shape[0], _dptr_words(out, "out"), _stream_handle(stream)))
    return out


class CrtKey:
    """A key of the approximate-CRT blind rotation (yg_crt_key_upload): the residue rows of the
    reference's BootstrappingKeyCRT::bsk8, int8 [n][4][2][2][2][N], on the torus Q_CRT."""

    def __init__(self, bsk8: np.ndarray, device: int = 0):
        a = np.ascontiguousarray(bsk8, np.int8)
        if a.ndim != 6 or a.shape[1:5] != (4, 2, 2, 2):
            raise ValueError("bsk8 must have shape [n, 4, 2, 2, 2, N]")
        self.n, self.N = a.shape[0], a.shape[-1]
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().yg_crt_key_upload(device, self.n, self.N, ctypes.c_void_p(a.ctypes.data),
                                                ctypes.byref(h)))
        self._h = h

    @property
    def device_bytes(self) -> int:
        return int(_lib.lib().yg_crt_key_device_bytes(self._h))

    def blind_rotate(self, acc_in, rot, out=None, stream=None):
        """blindRotateApproxCRTNtt with decompTrlweMcrt before and trlweMcrtToCrt +
        recompTrlweCrt after, per ciphertext: acc_in int32 [count, 2, N] (torus values mod
        Q_CRT), rot int32 [count, n]; returns the rotated samples int32 [count, 2, N]."""
        torch = _torch()
        if out is None:
            out = torch.empty_like(acc_in)
        _lib.check(_lib.lib().yg_crt_blind_rotate(self._h, _dptr(acc_in, "int32", "acc_in"), _dptr(rot, "int32", "rot"),
                                                  acc_in.shape[0], _dptr(out, "int32", "out"), _stream_handle(stream)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().yg_crt_key_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def blind_rotate_wwl24_ntt(ctx: Context, key: BootstrapKey, lwe_in, lut, steps: int | None = None, stream=None):
    """blindRotateWWL24Ntt (yatfhe/src/blind_rotate.cpp:1383-1412): the blind rotation on a
    WWL+24 key, whose GINX rows were derived on the GPU at upload."""
    if key.family != "wwl24":
        raise ValueError("blind_rotate_wwl24_ntt needs a key made by BootstrapKey.from_wwl24_words/_file")
    return blind_rotate_mp21_ntt(ctx, key, lwe_in, lut, steps=steps, stream=stream)


def blind_rotate_lazy_pipe_alt_ntt(ctx: Context, key: BootstrapKey, lwe_in, lut, stream=None):
    """blindRotateLazyPipeAltNtt (yatfhe/src/blind_rotate.cpp:995-1135) on a lazy key:
    accumulators [count, (k+1) N] (int64 torus words) after the whole rotation.  The
    reference's gdVntt argument (prepareGdV of the test polynomial) is computed on the GPU."""
    if key.family != "lazy":
        raise ValueError("blind_rotate_lazy_pipe_alt_ntt needs a key made by BootstrapKey.from_lazy_words/_file")
    return blind_rotate_mp21_ntt(ctx, key, lwe_in, lut, stream=stream)


def blind_rotate_ntt(ctx: Context, key: BootstrapKey, lwe_in, lut, stream=None):
    """blindRotateNtt (yatfhe/src/blind_rotate.cpp:549-560) after genNoiselessTrlweSample, on a
    group key: accumulators [count, (k+1) N] (int64 torus words) after the whole rotation."""
    if not key.family.startswith("group"):
        raise ValueError("blind_rotate_ntt needs a key made by BootstrapKey.from_group_words")
    return blind_rotate_mp21_ntt(ctx, key, lwe_in, lut, stream=stream)


def functional_bootstrapping_ntt(ctx: Context, key: BootstrapKey, lwe_in, lut, out=None, stream=None):
    """functionalBootstrappingNtt (yatfhe/src/bootstrapping.cpp:60-68) on a group key."""
    if not key.family.startswith("group"):
        raise ValueError("functional_bootstrapping_ntt needs a key made by BootstrapKey.from_group_words")
    return functional_bootstrapping_mp_ntt(ctx, key, lwe_in, lut, out=out, stream=stream)


def switch_key_for_tlwe(ctx: Context, key: BootstrapKey, big, stream=None):
    """Key-switches extracted ciphertexts ([count, kN+1] int32) to [count, n+1]."""
    torch = _torch()
    p = ctx.params
    out = torch.empty((big.shape[0], p.n + 1), dtype=torch.int32, device=big.device)
    _lib.check(_lib.lib().yg_keyswitch(ctx.handle, key.handle, _dptr(big, "int32", "big"), _dptr(out, "int32", "out"),
                                       big.shape[0], _stream_handle(stream)))
    return out
