"""Python access to the two CPU oracles.  TEST INFRASTRUCTURE ONLY.

* ``Restatement`` -- the plain-C restatement in oracle/pbs_oracle.c (built into
  oracle/_build/liboracle.so).  It needs nothing from the reference and runs anywhere.
* ``Reference``   -- the reference's own sources compiled against the stand-ins in
  oracle/shim (oracle/_ref/libyatfhe_ref_t{32,56}.so, built by ``make ref`` only where the
  reference tree exists).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs import
this module; the shipped package (yatfhe_gb300/) does not.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# The reference tree: $YATFHE_REFERENCE, else a checkout named "reference" beside this
# repository.  Absent on machines that only run the restatement.
REF_TREE = Path(os.environ.get("YATFHE_REFERENCE", HERE.parent.parent / "reference"))

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def _ptr(a: np.ndarray, typ):
    return a.ctypes.data_as(typ)


def build_restatement() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    return HERE / "_build" / "liboracle.so"


def reference_available() -> bool:
    return (REF_TREE / "yatfhe" / "src" / "bootstrapping.cpp").exists() or all(
        (HERE / "_ref" / f"libyatfhe_ref_t{t}.so").exists() for t in (32, 56))


def build_reference() -> None:
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "ref", f"REF={REF_TREE}"], check=True)


class _CParams(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int) for f in
                "n N k radix_bits l l_approx ks_radix_bits ks_level lwe_noise_b rlwe_noise_b torus_base torus_bits".split()]


def _cparams(p) -> _CParams:
    return _CParams(*(int(getattr(p, f)) for f, _ in _CParams._fields_))


class _Common:
    """Shared numpy-facing helpers; subclasses bind ``_call(name, *args)``."""

    p = None

    def _alloc_lwe(self, count):
        return np.zeros((count, self.p.n + 1), np.int32)

    def encrypt(self, mu) -> np.ndarray:
        mu = np.ascontiguousarray(mu, np.int64)
        out = self._alloc_lwe(len(mu))
        self._call("encrypt", _ptr(mu, _i64p), len(mu), _ptr(out, _i32p))
        return out

    def decrypt(self, lwe, base: int) -> np.ndarray:
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        out = np.zeros(len(lwe), np.int32)
        self._call("decrypt", _ptr(lwe, _i32p), len(lwe), base, _ptr(out, _i32p))
        return out

    def keys(self):
        s = np.zeros(self.p.n, np.int32)
        z = np.zeros(self.p.k * self.p.N, np.int32)
        self._call("get_keys" if self.prefix == "po_" else "export_keys", _ptr(s, _i32p), _ptr(z, _i32p))
        return s, z

    def ksk(self) -> np.ndarray:
        out = np.zeros(self.p.ksk_words if hasattr(self.p, "ksk_words") else
                       self.p.k * self.p.N * self.p.ks_level * (self.p.n + 1), np.int32)
        self._call("get_ksk" if self.prefix == "po_" else "export_ksk", _ptr(out, _i32p))
        return out

    def bsk_ntt(self) -> np.ndarray:
        p = self.p
        out = np.zeros(p.n * p.l_approx * (p.k + 1) ** 2 * p.N, np.uint64)
        self._call("get_bsk_ntt" if self.prefix == "po_" else "export_bsk_ntt", _ptr(out, _u64p))
        return out

    def test_polynomial(self, kind: int, modP: int) -> np.ndarray:
        v = np.zeros(self.p.N, np.int64)
        self._call("test_polynomial", kind, modP, _ptr(v, _i64p))
        return v

    def modswitch(self, lwe) -> np.ndarray:
        lwe = np.ascontiguousarray(lwe, np.int32)
        out = np.zeros(self.p.n + 1, np.int32)
        self._call("modswitch", _ptr(lwe, _i32p), _ptr(out, _i32p))
        return out

    def decompose(self, poly, levels: int) -> np.ndarray:
        poly = np.ascontiguousarray(poly, np.int64)
        out = np.zeros((levels, len(poly)), np.int64)
        if self.prefix == "po_":
            self._call("decompose", _ptr(poly, _i64p), levels, _ptr(out, _i64p))
        else:
            self._call("decompose", _ptr(poly, _i64p), len(poly), levels, _ptr(out, _i64p))
        return out

    def decompose_ks(self, value: int) -> np.ndarray:
        out = np.zeros(self.p.ks_level, np.int64)
        self._call("decompose_ks", ctypes.c_int64(int(value)), _ptr(out, _i64p))
        return out

    def ntt_forward(self, poly) -> np.ndarray:
        poly = np.ascontiguousarray(poly, np.int64)
        out = np.zeros(self.p.N, np.uint64)
        self._call("ntt_forward", _ptr(poly, _i64p), _ptr(out, _u64p))
        return out

    def ntt_inverse(self, ntt) -> np.ndarray:
        ntt = np.ascontiguousarray(ntt, np.uint64)
        out = np.zeros(self.p.N, np.int64)
        self._call("ntt_inverse", _ptr(ntt, _u64p), _ptr(out, _i64p))
        return out

    def external_product(self, trlwe, i: int) -> np.ndarray:
        trlwe = np.ascontiguousarray(trlwe, np.int64)
        out = np.zeros_like(trlwe)
        self._call("external_product", _ptr(trlwe, _i64p), i, _ptr(out, _i64p))
        return out

    def extract(self, acc) -> np.ndarray:
        acc = np.ascontiguousarray(acc, np.int64)
        out = np.zeros(self.p.k * self.p.N + 1, np.int32)
        self._call("extract", _ptr(acc, _i64p), _ptr(out, _i32p))
        return out

    def keyswitch(self, lwe_big) -> np.ndarray:
        lwe_big = np.ascontiguousarray(lwe_big, np.int32)
        out = np.zeros(self.p.n + 1, np.int32)
        self._call("keyswitch", _ptr(lwe_big, _i32p), _ptr(out, _i32p))
        return out

    def blind_rotate_trace(self, lwe, v, checkpoints):
        lwe = np.ascontiguousarray(lwe, np.int32)
        v = np.ascontiguousarray(v, np.int64)
        cps = np.ascontiguousarray(sorted(checkpoints), np.int32)
        stride = (self.p.k + 1) * self.p.N
        out = np.zeros((len(cps), stride), np.int64)
        final = np.zeros(stride, np.int64)
        self._call("blind_rotate_trace", _ptr(lwe, _i32p), _ptr(v, _i64p),
                   cps.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(cps), _ptr(out, _i64p),
                   _ptr(final, _i64p))
        return out, final

    def pbs(self, lwe, v, threads: int = 1) -> np.ndarray:
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        out = np.zeros_like(lwe)
        self._call("pbs", _ptr(lwe, _i32p), len(lwe), _ptr(v, _i64p), _ptr(out, _i32p), threads)
        return out

    # WWL+24 keys: cprime [n][l_approx][k+1][N] and s2 [l][k+1][N] NTT-domain words.
    def keygen_wwl24(self, seed: int) -> None:
        self._call("keygen_wwl24", ctypes.c_uint64(seed))

    def wwl24_words(self):
        p = self.p
        cprime = np.zeros((p.n, p.l_approx, p.k + 1, p.N), np.uint64)
        s2 = np.zeros((p.l, p.k + 1, p.N), np.uint64)
        self._call("get_wwl24" if self.prefix == "po_" else "export_wwl24", _ptr(cprime, _u64p), _ptr(s2, _u64p))
        return cprime, s2

    def wwl24_expanded(self) -> np.ndarray:
        """The GINX rows blindRotateWWL24Ntt derives from the WWL+24 key, [n][l_approx][k+1][k+1][N]
        (the layout of bsk_ntt())."""
        p = self.p
        if self.prefix == "po_":
            self._call("wwl24_expand")
            return self.bsk_ntt()
        out = np.zeros(p.n * p.l_approx * (p.k + 1) ** 2 * p.N, np.uint64)
        self._call("wwl24_expand", _ptr(out, _u64p))
        return out


    # Lazy keys: cprime [n][l_approx][k+1][N] coefficient-domain torus values, s2 [l][k+1][N]
    # NTT-domain words.
    def keygen_lazy(self, seed: int) -> None:
        self._call("keygen_lazy", ctypes.c_uint64(seed))

    def lazy_words(self):
        p = self.p
        cprime = np.zeros((p.n, p.l_approx, p.k + 1, p.N), np.int64)
        s2 = np.zeros((p.l, p.k + 1, p.N), np.uint64)
        self._call("get_lazy" if self.prefix == "po_" else "export_lazy", _ptr(cprime, _i64p), _ptr(s2, _u64p))
        return cprime, s2


    # Group-g keys of blindRotateNtt: TrgswDft words [keys][l][k+1][k+1][N].
    def group_key_count(self, group: int) -> int:
        return self.p.n if group == 1 else (self.p.n // group) << group

    def keygen_group(self, seed: int, group: int) -> None:
        self._call("keygen_group", ctypes.c_uint64(seed), group)
        self._group = group

    def group_words(self) -> np.ndarray:
        p, g = self.p, self._group
        out = np.zeros((self.group_key_count(g), p.l, p.k + 1, p.k + 1, p.N), np.uint64)
        self._call("get_group" if self.prefix == "po_" else "export_group", _ptr(out, _u64p))
        return out


class Restatement(_Common):
    """The plain-C oracle for one parameter set."""

    prefix = "po_"
    _lib = None

    @staticmethod
    def load():
        if Restatement._lib is None:
            so = HERE / "_build" / "liboracle.so"
            if not so.exists():
                build_restatement()
            Restatement._lib = ctypes.CDLL(str(so))
            Restatement._lib.po_create.restype = ctypes.c_void_p
            Restatement._lib.po_last_error.restype = ctypes.c_char_p
            Restatement._lib.po_last_error.argtypes = [ctypes.c_void_p]
            Restatement._lib.po_destroy.argtypes = [ctypes.c_void_p]
            Restatement._lib.po_qntt.restype = ctypes.c_uint64
            Restatement._lib.po_qntt.argtypes = [ctypes.c_void_p]
        return Restatement._lib

    def __init__(self, p):
        Restatement.load()
        self.p = p
        cp = _cparams(p)
        self._h = Restatement._lib.po_create(ctypes.byref(cp))
        if not self._h:
            raise ValueError(f"po_create rejected {p}")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and Restatement._lib is not None:
            Restatement._lib.po_destroy(h)
            self._h = None

    def _call(self, name, *args):
        fn = getattr(Restatement._lib, "po_" + name)
        rc = fn(ctypes.c_void_p(self._h), *args)
        if rc != 0:
            raise RuntimeError(f"po_{name}: {Restatement._lib.po_last_error(self._h).decode()}")

    def keygen(self, seed: int) -> None:
        self._call("keygen", ctypes.c_uint64(seed))

    def set_keys(self, lwe_s, rlwe_s) -> None:
        a = np.ascontiguousarray(lwe_s, np.int32)
        b = np.ascontiguousarray(rlwe_s, np.int32)
        self._call("set_keys", _ptr(a, _i32p), _ptr(b, _i32p))

    def set_ksk(self, ksk) -> None:
        a = np.ascontiguousarray(ksk, np.int32)
        self._call("set_ksk", _ptr(a, _i32p))

    def set_bsk_ntt(self, bsk) -> None:
        a = np.ascontiguousarray(bsk, np.uint64)
        self._call("set_bsk_ntt", _ptr(a, _u64p))

    def save_bsk_file(self, path) -> None:
        self._call("save_bsk_file", str(path).encode())

    def load_bsk_file(self, path) -> None:
        self._call("load_bsk_file", str(path).encode())

    def encrypt_samples(self, mu):
        """encrypt(mu) that also returns each ciphertext's mask [count][n] and noise [count]."""
        mu = np.ascontiguousarray(mu, np.int64)
        out = self._alloc_lwe(len(mu))
        mask = np.zeros((len(mu), self.p.n), np.int32)
        noise = np.zeros(len(mu), np.int32)
        self._call("encrypt_samples", _ptr(mu, _i64p), len(mu), _ptr(out, _i32p), _ptr(mask, _i32p),
                   _ptr(noise, _i32p))
        return out, mask, noise

    def encrypt_rlwe_ntt_samples(self, mu):
        """NTT-domain RLWE encryptions of the torus polynomials mu [count][N]: the samples
        [count][k+1][N] (uint64 mod q) with their masks [count][k][N] and noise [count][N]."""
        p = self.p
        mu = np.ascontiguousarray(mu, np.int64).reshape(-1, p.N)
        out = np.zeros((len(mu), p.k + 1, p.N), np.uint64)
        mask = np.zeros((len(mu), p.k, p.N), np.uint64)
        noise = np.zeros((len(mu), p.N), np.int32)
        self._call("encrypt_rlwe_ntt_samples", _ptr(mu, _i64p), len(mu), _ptr(out, _u64p), _ptr(mask, _u64p),
                   _ptr(noise, _i32p))
        return out, mask, noise

    def keygen_samples(self, seed: int) -> dict:
        """keygen(seed) that also returns its random samples: the secrets, the BSK samples'
        noise [n][l][k+1][N] and masks [n][l][k+1][k][N], the KSK samples' masks [kN][t][n]
        and noise [kN][t]."""
        p = self.p
        k1, kN = p.k + 1, p.k * p.N
        d = {"lwe_s": np.zeros(p.n, np.int32), "rlwe_s": np.zeros(kN, np.int32),
             "bsk_noise": np.zeros((p.n, p.l_approx, k1, p.N), np.int32),
             "bsk_mask": np.zeros((p.n, p.l_approx, k1, p.k, p.N), np.uint64),
             "ksk_mask": np.zeros((kN, p.ks_level, p.n), np.int32),
             "ksk_noise": np.zeros((kN, p.ks_level), np.int32)}
        self._call("keygen_samples", ctypes.c_uint64(seed), _ptr(d["lwe_s"], _i32p), _ptr(d["rlwe_s"], _i32p),
                   _ptr(d["bsk_noise"], _i32p), _ptr(d["bsk_mask"], _u64p), _ptr(d["ksk_mask"], _i32p),
                   _ptr(d["ksk_noise"], _i32p))
        return d

    def set_wwl24(self, cprime, s2) -> None:
        a = np.ascontiguousarray(cprime, np.uint64)
        b = np.ascontiguousarray(s2, np.uint64)
        self._call("set_wwl24", _ptr(a, _u64p), _ptr(b, _u64p))

    def save_wwl24_file(self, path) -> None:
        self._call("save_wwl24_file", str(path).encode())

    def load_wwl24_file(self, path) -> None:
        self._call("load_wwl24_file", str(path).encode())

    def pbs_wwl24(self, lwe, v, threads: int = 1) -> np.ndarray:
        """The WWL+24 bootstrap: the GINX bootstrap on the expanded key."""
        self._call("wwl24_expand")
        return self.pbs(lwe, v, threads)

    def set_lazy(self, cprime, s2) -> None:
        a = np.ascontiguousarray(cprime, np.int64)
        b = np.ascontiguousarray(s2, np.uint64)
        self._call("set_lazy", _ptr(a, _i64p), _ptr(b, _u64p))

    def set_group(self, words, group: int) -> None:
        a = np.ascontiguousarray(words, np.uint64)
        self._call("set_group", _ptr(a, _u64p), group)
        self._group = group

    def blind_rotate_group(self, lwe, v) -> np.ndarray:
        """The accumulator [(k+1) N] after blindRotateNtt on the group key, one ciphertext."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        acc = np.zeros((self.p.k + 1) * self.p.N, np.int64)
        self._call("blind_rotate_group", _ptr(lwe, _i32p), _ptr(v, _i64p), _ptr(acc, _i64p))
        return acc

    def pbs_group(self, lwe, v, threads: int = 1) -> np.ndarray:
        """functionalBootstrappingNtt on the group key."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        out = np.zeros_like(lwe)
        self._call("pbs_group", _ptr(lwe, _i32p), len(lwe), _ptr(v, _i64p), _ptr(out, _i32p), threads)
        return out

    def save_lazy_file(self, path) -> None:
        self._call("save_lazy_file", str(path).encode())

    def load_lazy_file(self, path) -> None:
        self._call("load_lazy_file", str(path).encode())

    def blind_rotate_lazy(self, lwe, v, no_first: bool = False) -> np.ndarray:
        """The accumulator [(k+1) N] after the lazy blind rotation of one ciphertext
        (blindRotateLazyPipeAltNtt, or with no_first blindRotateLazyPipeAltNoFirstNtt)."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        acc = np.zeros((self.p.k + 1) * self.p.N, np.int64)
        self._call("blind_rotate_lazy_no_first" if no_first else "blind_rotate_lazy", _ptr(lwe, _i32p),
                   _ptr(v, _i64p), _ptr(acc, _i64p))
        return acc

    def pbs_lazy(self, lwe, v, threads: int = 1, no_first: bool = False) -> np.ndarray:
        """The bootstrap with blindRotateLazyPipeAltNtt (or NoFirstNtt) on the lazy key."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        out = np.zeros_like(lwe)
        self._call("pbs_lazy_no_first" if no_first else "pbs_lazy", _ptr(lwe, _i32p), len(lwe), _ptr(v, _i64p),
                   _ptr(out, _i32p), threads)
        return out

    @property
    def q(self) -> int:
        return int(Restatement._lib.po_qntt(self._h))


class Reference(_Common):
    """The reference's own code (one process-global parameter set per torus build)."""

    prefix = "ref_"
    _libs: dict = {}

    def __init__(self, p):
        t = p.torus_bits
        if t not in Reference._libs:
            so = HERE / "_ref" / f"libyatfhe_ref_t{t}.so"
            if not so.exists():
                build_reference()
            lib = ctypes.CDLL(str(so))
            lib.ref_last_error.restype = ctypes.c_char_p
            lib.ref_ntt_root.restype = ctypes.c_uint64
            Reference._libs[t] = lib
        self.lib = Reference._libs[t]
        self.p = p
        cp = _CParams(*(int(getattr(p, f)) for f, _ in _CParams._fields_))
        if self.lib.ref_setup(ctypes.byref(cp)) != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())

    def _call(self, name, *args):
        rc = getattr(self.lib, "ref_" + name)(*args)
        if rc != 0:
            raise RuntimeError(f"ref_{name}: {self.lib.ref_last_error().decode()}")

    def keygen(self, seed: int) -> None:
        self._call("keygen", ctypes.c_uint64(seed))

    def save_bsk_file(self, path) -> None:
        self._call("save_bsk", str(path).encode())

    def load_bsk_file(self, path) -> None:
        self._call("load_bsk", str(path).encode())

    def save_wwl24_file(self, path) -> None:
        self._call("save_wwl24", str(path).encode())

    def load_wwl24_file(self, path) -> None:
        self._call("load_wwl24", str(path).encode())

    def pbs_wwl24(self, lwe, v, with_acc: bool = False):
        """functionalBootstrappingMPNtt's composition around blindRotateWWL24Ntt; with_acc also
        returns ciphertext 0's accumulator after the blind rotation."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        out = np.zeros_like(lwe)
        acc = np.zeros((self.p.k + 1) * self.p.N, np.int64)
        self._call("pbs_wwl24", _ptr(lwe, _i32p), len(lwe), _ptr(v, _i64p), _ptr(out, _i32p), _ptr(acc, _i64p))
        return (out, acc) if with_acc else out

    def pbs_group(self, lwe, v, with_acc: bool = False):
        """functionalBootstrappingNtt's composition on the group key; with_acc also returns
        ciphertext 0's accumulator after blindRotateNtt."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        out = np.zeros_like(lwe)
        acc = np.zeros((self.p.k + 1) * self.p.N, np.int64)
        self._call("pbs_group", _ptr(lwe, _i32p), len(lwe), _ptr(v, _i64p), _ptr(out, _i32p), _ptr(acc, _i64p))
        return (out, acc) if with_acc else out

    def save_lazy_file(self, path) -> None:
        self._call("save_lazy", str(path).encode())

    def load_lazy_file(self, path) -> None:
        self._call("load_lazy", str(path).encode())

    def pbs_lazy(self, lwe, v, with_acc: bool = False, no_first: bool = False):
        """functionalBootstrappingMPNtt's composition around blindRotateLazyPipeAltNtt (or, with
        no_first, blindRotateLazyPipeAltNoFirstNtt); with_acc also returns ciphertext 0's
        accumulator after the blind rotation."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        out = np.zeros_like(lwe)
        acc = np.zeros((self.p.k + 1) * self.p.N, np.int64)
        self._call("pbs_lazy_no_first" if no_first else "pbs_lazy", _ptr(lwe, _i32p), len(lwe), _ptr(v, _i64p),
                   _ptr(out, _i32p), _ptr(acc, _i64p))
        return (out, acc) if with_acc else out

    def pbs_lazy_sweep(self, lwe, v, move_ntt: int, units_a: int) -> np.ndarray:
        """ref_pbs_lazy with blindRotateLazyPipeAltNttSweep's pipeline split."""
        lwe = np.ascontiguousarray(lwe, np.int32).reshape(-1, self.p.n + 1)
        v = np.ascontiguousarray(v, np.int64)
        out = np.zeros_like(lwe)
        self._call("pbs_lazy_sweep", _ptr(lwe, _i32p), len(lwe), _ptr(v, _i64p), _ptr(out, _i32p), move_ntt, units_a)
        return out

    def set_keys(self, lwe_s, rlwe_s) -> None:
        a = np.ascontiguousarray(lwe_s, np.int32)
        b = np.ascontiguousarray(rlwe_s, np.int32)
        self._call("import_keys", _ptr(a, _i32p), _ptr(b, _i32p))

    def set_ksk(self, ksk) -> None:
        a = np.ascontiguousarray(ksk, np.int32)
        self._call("import_ksk", _ptr(a, _i32p))

    def rotate(self, poly, a: int, minus_one: bool) -> np.ndarray:
        poly = np.ascontiguousarray(poly, np.int64)
        out = np.zeros_like(poly)
        self._call("rotate", _ptr(poly, _i64p), len(poly), a, int(minus_one), _ptr(out, _i64p))
        return out

    def pbs_pool(self, lwe, v) -> np.ndarray:
        """One reference-ThreadPool task per ciphertext (throughput form)."""
        return self.pbs(lwe, v, threads=1)

    def ntt_root(self) -> int:
        return int(self.lib.ref_ntt_root())


def _restatement_rotate(self, poly, a: int, minus_one: bool) -> np.ndarray:
    poly = np.ascontiguousarray(poly, np.int64)
    out = np.zeros_like(poly)
    self._call("rotate", _ptr(poly, _i64p), a, int(minus_one), _ptr(out, _i64p))
    return out


Restatement.rotate = _restatement_rotate


# ------------------------------------------------------------------ approximate CRT

CRT_PRIMES = (251, 241, 239, 233)
CRT_Q = 251 * 241 * 239 * 233


def crt_blind_rotate(bsk8, acc_in, rot):
    """The restatement of blindRotateApproxCRTNtt with its conversions (po_crt_blind_rotate):
    bsk8 int8 [n][4][2][2][2][N], acc_in torus values mod Q_CRT [2][N], rot [n].  Returns the
    rotated sample [2][N] (int64) and the residue samples after the rotation [4][2][N] (int8)."""
    bsk8 = np.ascontiguousarray(bsk8, np.int8)
    n, N = bsk8.shape[0], bsk8.shape[-1]
    acc_in = np.ascontiguousarray(acc_in, np.int64).reshape(2, N)
    rot = np.ascontiguousarray(rot, np.int32).reshape(n)
    out = np.zeros((2, N), np.int64)
    mcrt = np.zeros((4, 2, N), np.int8)
    rc = Restatement.load().po_crt_blind_rotate(n, N, _ptr(bsk8, ctypes.c_void_p), _ptr(acc_in, _i64p),
                                                _ptr(rot, _i32p), _ptr(out, _i64p), _ptr(mcrt, ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError("po_crt_blind_rotate failed")
    return out, mcrt


class CrtReference:
    """The reference's ApproxCRT path (ref_crt_*, T32 build): keys, encryption, decryption and
    the blind rotation, process-global like Reference."""

    def __init__(self, n: int, N: int, rlwe_noise_b: int = 3, torus_base: int = 4):
        so = HERE / "_ref" / "libyatfhe_ref_t32.so"
        if not so.exists():
            build_reference()
        if 32 not in Reference._libs:
            lib = ctypes.CDLL(str(so))
            lib.ref_last_error.restype = ctypes.c_char_p
            lib.ref_ntt_root.restype = ctypes.c_uint64
            Reference._libs[32] = lib
        self.lib = Reference._libs[32]
        self.n, self.N, self.base = n, N, torus_base
        if self.lib.ref_crt_setup(n, N, rlwe_noise_b, torus_base) != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())

    def _call(self, name, *args):
        if getattr(self.lib, "ref_crt_" + name)(*args) != 0:
            raise RuntimeError(f"ref_crt_{name}: {self.lib.ref_last_error().decode()}")

    def keygen(self, seed: int):
        self._call("keygen", ctypes.c_uint64(seed))

    def bsk8(self) -> np.ndarray:
        out = np.zeros((self.n, 4, 2, 2, 2, self.N), np.int8)
        self._call("export_bsk8", _ptr(out, ctypes.c_void_p))
        return out

    def set_bsk8(self, bsk8) -> None:
        a = np.ascontiguousarray(bsk8, np.int8)
        self._call("import_bsk8", _ptr(a, ctypes.c_void_p))

    def lwe_key(self) -> np.ndarray:
        s = np.zeros(self.n, np.int32)
        z = np.zeros(self.N, np.int32)
        if self.lib.ref_export_keys(_ptr(s, _i32p), _ptr(z, _i32p)) != 0:
            raise RuntimeError(self.lib.ref_last_error().decode())
        return s

    def encrypt(self, plain) -> np.ndarray:
        plain = np.ascontiguousarray(plain, np.int32)
        out = np.zeros((2, self.N), np.int64)
        self._call("encrypt", _ptr(plain, _i32p), _ptr(out, _i64p))
        return out

    def decrypt(self, acc) -> np.ndarray:
        acc = np.ascontiguousarray(acc, np.int64)
        out = np.zeros(self.N, np.int32)
        self._call("decrypt", _ptr(acc, _i64p), _ptr(out, _i32p))
        return out

    def blind_rotate(self, acc_in, rot, ntt: bool = True):
        acc_in = np.ascontiguousarray(acc_in, np.int64)
        rot = np.ascontiguousarray(rot, np.int32)
        out = np.zeros((2, self.N), np.int64)
        mcrt = np.zeros((4, 2, self.N), np.int8)
        self._call("blind_rotate", _ptr(acc_in, _i64p), _ptr(rot, _i32p), int(ntt), _ptr(out, _i64p),
                   _ptr(mcrt, ctypes.c_void_p))
        return out, mcrt
