"""ctypes binding of libhora_gb300.so (include/hora_gb300.h).

Loading fails loudly when the shared library is missing: there is no CPU
fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "libhora_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "hora_gb300.h")

OK = 0
ERRORS = {
    -1: "EINVAL", -2: "EDIM", -3: "ECAP", -4: "EMETRIC", -5: "ENAN", -6: "EOOM", -7: "ECUDA",
    -8: "ENOTBUILT", -9: "ENOTIMPL", -10: "EIO", -11: "ETIMEDOUT", -12: "ESIZE",
}


class HoraError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code
        self.msg = msg


class IVFPQParamsC(C.Structure):
    _fields_ = [("n_sub", C.c_uint64), ("sub_bits", C.c_uint64), ("n_kmeans_center", C.c_uint64),
                ("search_n_center", C.c_uint64), ("train_epoch", C.c_uint64)]


class PQParamsC(C.Structure):
    _fields_ = [("n_sub", C.c_uint64), ("sub_bits", C.c_uint64), ("train_epoch", C.c_uint64)]


_lib = None

vp = C.c_void_p
u64 = C.c_uint64
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)
i64p = C.POINTER(C.c_int64)
u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
f64p = C.POINTER(C.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "hora_last_error": (C.c_char_p, []),
    "hora_version": (C.c_char_p, []),
    "hora_kernel_launches": (u64, []),
    "hora_profile_enable": (C.c_int, [C.c_int]),
    "hora_profile_report": (C.c_int, [C.c_char_p, u64]),
    "hora_ivfpq_params_default": (None, [C.POINTER(IVFPQParamsC)]),
    "hora_pq_params_default": (None, [C.POINTER(PQParamsC)]),
    "hora_load_reference": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(vp)]),
    "hora_knn_graph": (C.c_int, [vp, u64, vp]),
    "hora_general_kmeans": (C.c_int, [vp, u64, u64, vp, u64, vp, vp]),
    "hora_index_create": (C.c_int, [C.c_int, u64, vp, C.POINTER(vp)]),
    "hora_index_free": (C.c_int, [vp]),
    "hora_add": (C.c_int, [vp, vp, vp, u64]),
    "hora_build": (C.c_int, [vp, C.c_int]),
    "hora_built": (C.c_int, [vp, C.POINTER(C.c_int)]),
    "hora_rebuild": (C.c_int, [vp, C.c_int]),
    "hora_search": (C.c_int, [vp, vp, u64, u64, vp, vp]),
    "hora_search_nodes": (C.c_int, [vp, vp, u64, u64, vp, vp, vp]),
    "hora_search_nprobe": (C.c_int, [vp, vp, u64, u64, u64, vp, vp]),
    "hora_name": (C.c_int, [vp, C.POINTER(C.c_char_p)]),
    "hora_nodes_size": (C.c_int, [vp, u64p]),
    "hora_dimension": (C.c_int, [vp, u64p]),
    "hora_clear": (C.c_int, [vp]),
    "hora_idx_info": (C.c_int, [vp, C.c_char_p, u64]),
    "hora_dump": (C.c_int, [vp, C.c_char_p]),
    "hora_load": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "hora_set_option": (C.c_int, [vp, C.c_int, C.c_double]),
    "hora_get_option": (C.c_int, [vp, C.c_int, f64p]),
    "hora_ivfpq_layout": (C.c_int, [vp, u64p, u64p, u64p, u64p]),
    "hora_ivfpq_export": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "hora_ivfpq_set_codebooks": (C.c_int, [vp, vp, vp]),
    "hora_ivfpq_train_nprobe": (C.c_int, [vp, vp, u64, u64, C.c_double, u64, f64p]),
    "hora_ivfpq_nprobe_features": (C.c_int, [vp, vp, u64, vp]),
    "hora_ivfpq_predict_nprobe": (C.c_int, [vp, vp, u64, vp]),
    "hora_mlp_forward": (C.c_int, [vp, u64, u64, u64, vp, u64, vp]),
    "hora_mlp_loss_grad": (C.c_int, [vp, u64, u64, u64, vp, vp, u64, C.c_float, vp, vp]),
    "hora_server_create": (C.c_int, [C.POINTER(vp), C.c_uint32, C.c_uint32, u64, C.POINTER(vp)]),
    "hora_server_free": (C.c_int, [vp]),
    "hora_server_submit": (C.c_int, [vp, C.c_uint32, vp, u64, u64, vp, vp, u64p]),
    "hora_server_wait": (C.c_int, [vp, u64, C.c_int64, f64p]),
    "hora_server_stats": (C.c_int, [vp, f64p]),
    "hora_server_request_bytes": (C.c_int, [vp, C.c_uint32, u64, u64, u64p]),
    "hora_server_info": (C.c_int, [vp, C.c_char_p, u64]),
    "hora_bf_search_noalloc": (C.c_int, [vp, u64, u64, vp, u64, u64, C.c_int, vp, vp, vp]),
}


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    txt = open(HEADER).read()
    pat = r"^\s*(?:const\s+)?(?:int|void|char|uint64_t)\s*\*?\s*(hora_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(pat, txt, flags=re.M)))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(SO):
            raise ImportError(
                f"{SO} is missing: build it with `python -m hora_gb300.build` "
                "(there is no CPU fallback)")
        L = C.CDLL(SO)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != OK:
        raise HoraError(rc, lib().hora_last_error().decode())


def launches() -> int:
    return int(lib().hora_kernel_launches())


def profile(on: bool) -> None:
    lib().hora_profile_enable(1 if on else 0)


def profile_report() -> dict:
    """{kernel name: (launches, total ms)} since the last report."""
    import json
    buf = C.create_string_buffer(1 << 16)
    check(lib().hora_profile_report(buf, len(buf)))
    return {k: (int(v[0]), float(v[1])) for k, v in json.loads(buf.value.decode()).items()}
