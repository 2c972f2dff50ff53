"""CPU tests of the C ABI: the library builds, loads and exports every symbol
the public header declares.  No compute call is made (no GPU here)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_header_symbols(hora):
    from hora_gb300 import _lib
    L = C.CDLL(_lib.SO)
    names = _lib.header_symbols()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert not [n for n in names if n not in _lib.SIGNATURES]


def test_option_keys_match_header(hora):
    """The Python Option enum carries every hora_option key of the header
    with the same value."""
    import re
    from hora_gb300 import _lib
    txt = open(_lib.HEADER).read()
    body = txt[txt.index("HORA_OPT_PRECISION"):txt.index("} hora_option;")]
    keys = {m.group(1): int(m.group(2)) for m in re.finditer(r"HORA_OPT_([A-Z0-9_]+)\s*=\s*(\d+)", body)}
    assert len(keys) >= 12
    assert keys == {o.name: int(o.value) for o in hora.Option}


def test_version_and_error_string(hora):
    L = hora.lib()
    assert b"sm_103a" in L.hora_version()
    assert isinstance(L.hora_last_error(), bytes)


def test_null_arguments_fail_cleanly(hora):
    L = hora.lib()
    assert L.hora_index_create(0, 4, None, None) == -1
    assert L.hora_add(None, None, None, 1) == -1
    assert b"null" in L.hora_last_error()
    assert L.hora_rebuild(None, 3) == -9  # "not implement" (ann_index.rs:69-71)


def test_params_default_matches_reference(hora):
    from hora_gb300._lib import IVFPQParamsC
    p = IVFPQParamsC()
    hora.lib().hora_ivfpq_params_default(C.byref(p))
    # IVFPQParams::default (src/index/pq_params.rs:80-91)
    assert (p.n_sub, p.sub_bits, p.n_kmeans_center, p.search_n_center, p.train_epoch) == \
        (25, 4, 256, 8, 100)


def test_pq_params_default_matches_reference(hora):
    from hora_gb300._lib import PQParamsC
    p = PQParamsC()
    hora.lib().hora_pq_params_default(C.byref(p))
    # PQParams::default (src/index/pq_params.rs:32-41)
    assert (p.n_sub, p.sub_bits, p.train_epoch) == (4, 4, 100)


def test_reference_file_parse_errors_fail_cleanly(hora, tmp_path):
    # a truncated or malformed bincode file is rejected while parsing, before
    # any device work (hora_load_reference)
    from tests import refbin
    X = np.arange(40, dtype=np.float32).reshape(10, 4)
    good = refbin.brute_force(X, list(range(10)), 3)
    L = hora.lib()
    h = C.c_void_p()
    for blob in (good[:-3], good[:20], b"", good[:8] + b"\xff" * 8 + good[16:]):
        p = tmp_path / "bad.bin"
        p.write_bytes(blob)
        assert L.hora_load_reference(str(p).encode(), 0, C.byref(h)) == -10  # HORA_EIO
        assert not h.value
    assert L.hora_load_reference(b"/nonexistent/file", 0, C.byref(h)) == -10
    assert L.hora_load_reference(str(tmp_path / "bad.bin").encode(), 7, C.byref(h)) == -1


def test_cpp_wrapper_compiles():
    """include/hora_gb300.hpp (the ANNIndex-shaped C++ wrapper) compiles."""
    src = os.path.join(ROOT, "include", "hora_gb300.hpp")
    if not os.path.exists(src):
        pytest.skip("no C++ wrapper")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-x", "c++", src], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr


def test_no_cpu_fallback_in_package():
    """The product package never imports or links the oracle."""
    pkg = os.path.join(ROOT, "hora_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cpp", ".h", ".cuh")):
                txt = open(os.path.join(dirpath, f)).read()
                for bad in ("import oracle", "from oracle", "hora_oracle", "horo_"):
                    assert bad not in txt, (f, bad)
