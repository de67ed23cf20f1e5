"""CPU checks of the C ABI: the library builds for sm_103a, loads without a GPU, and
exports every function include/yatfhe_gb300.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared(header: Path) -> set[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(yg_[a-z0-9_]+)\s*\(", text))


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    declared = set()
    for h in (ROOT / "include").glob("*.h"):
        declared |= _declared(h)
    assert declared, "no declarations found"
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_the_header(built_lib):
    from yatfhe_gb300 import _lib

    declared = set()
    for h in (ROOT / "include").glob("*.h"):
        declared |= _declared(h)
    assert declared == set(_lib.exported_symbols())


def test_last_error_is_empty_initially(built_lib):
    from yatfhe_gb300 import _lib

    assert _lib.lib().yg_last_error() in (b"",)


def test_invalid_parameters_are_rejected_before_any_device_work(built_lib):
    """Parameter validation runs on the host (std::invalid_argument -> YG_ERR_INVALID)."""
    from yatfhe_gb300 import _lib
    from yatfhe_gb300.params import T32_N1024

    bad = [
        dict(torus_bits=40),
        dict(N=512),
        dict(k=2),
        dict(l_approx=5, radix_bits=7),   # 35 bits > T = 32
        dict(ks_level=17, ks_radix_bits=1),
        dict(radix_bits=16, l_approx=2),
        dict(radix_bits=1, l_approx=16),  # 64-bit channel-row sums need l <= 15
    ]
    for change in bad:
        fields = {f: getattr(T32_N1024, f) for f in ("n", "N", "k", "radix_bits", "l_approx", "ks_radix_bits",
                                                     "ks_level", "torus_bits")}
        fields.update(change)
        prm = _lib.YgParams(*fields.values())
        h = ctypes.c_void_p()
        rc = _lib.lib().yg_ctx_create(ctypes.byref(prm), 0, ctypes.byref(h))
        assert rc == -1, change
        assert _lib.lib().yg_last_error()


def test_null_arguments_are_rejected(built_lib):
    from yatfhe_gb300 import _lib

    L = _lib.lib()
    assert L.yg_ctx_create(None, 0, None) == -1
    assert L.yg_pbs(None, None, None, None, 1, None, None) == -1
    assert L.yg_key_upload_wwl24_ntt(None, None, None, 1, None) == -1
    assert L.yg_key_load_wwl24_file(None, None, None) == -1
    assert L.yg_key_upload_lazy(None, None, None, 1, None) == -1
    assert L.yg_key_load_lazy_file(None, None, None) == -1
    assert L.yg_key_upload_group(None, None, 2, 3, None) == -1
    assert L.yg_key_device_bytes(None) == 0
    L.yg_ctx_destroy(None)
    L.yg_key_destroy(None)


def test_product_does_not_import_the_oracle():
    """The shipped package never imports, links or runs anything under oracle/."""
    for f in (ROOT / "yatfhe_gb300").rglob("*"):
        if f.suffix in (".py", ".cu", ".cuh", ".cpp", ".h", ".hpp"):
            text = f.read_text()
            assert "oracle" not in re.sub(r"(#|//).*", "", text).lower() or f.name == "__init__.py", f


STRUCTS = {  # ctypes mirror in yatfhe_gb300/_lib.py -> C struct in include/yatfhe_gb300.h
    "YgParams": "yg_params",
    "ServerConfig": "yg_server_config",
    "ServerCounters": "yg_server_counters",
    "RequestTimes": "yg_request_times",
    "TraceConfig": "yg_trace_config",
    "Latency": "yg_latency",
    "TraceResult": "yg_trace_result",
}


def test_ctypes_structs_match_the_header(tmp_path):
    """Every struct the Python binding passes through the C ABI has the header's size and
    field offsets (a probe compiled with the host C compiler prints them)."""
    import shutil
    import subprocess

    from yatfhe_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "yatfhe_gb300.h"', "int main(void) {"]
    for py, c in STRUCTS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for f, _ in getattr(_lib, py)._fields_:
            lines.append(f'  printf("{py} {f} %zu\\n", offsetof({c}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for py in STRUCTS:
        cls = getattr(_lib, py)
        assert got[(py, "size")] == ctypes.sizeof(cls), py
        for f, _ in cls._fields_:
            assert got[(py, f)] == getattr(cls, f).offset, (py, f)


def test_layout_constants_match_the_header():
    from yatfhe_gb300 import _lib

    text = (ROOT / "include" / "yatfhe_gb300.h").read_text()
    defined = dict(re.findall(r"#define (YG_LAYOUT_[A-Z_]+) (\d+)", text))
    assert defined, "no layout constants found"
    for name, value in defined.items():
        assert getattr(_lib, name[len("YG_"):]) == int(value), name
