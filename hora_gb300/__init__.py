"""hora_gb300 — GB300 (sm_103a) implementation of hora's data-parallel search
path: brute-force k-NN over the four metrics and IVF-PQ build and search,
behind a C ABI that mirrors hora's ANNIndex trait (include/hora_gb300.h).

The compute runs in libhora_gb300.so (hand-written CUDA); this package is the
thin host-side mirror of the reference's API.  It raises ImportError-style
errors when the library is missing; there is no CPU fallback.
"""
from ._lib import HoraError, launches, lib  # noqa: F401
from .index import (NO_ID, BruteForceIndex, BruteForceParams, IVFPQIndex,  # noqa: F401
                    IVFPQParams, Metric, Node, Option, PQIndex, PQIVFIndex, PQParams, Precision,
                    Server, load_reference)

__all__ = ["BruteForceIndex", "BruteForceParams", "IVFPQIndex", "PQIVFIndex", "IVFPQParams",
           "PQIndex", "PQParams", "load_reference",
           "Metric", "Node", "Option", "Precision", "Server", "HoraError", "NO_ID", "lib", "launches"]
