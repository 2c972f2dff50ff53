"""Seeded synthetic workloads with the shapes and distributions of the
benchmark configurations (the ann-benchmarks datasets the reference plots are
not available offline, so these stand in for them).

- normal(n, d, sigma):  i.i.d. Normal(0, sigma) entries
  (examples/src/demo.rs:11 uses Normal(0, 10)).
- mixture(n, d, centers): Gaussian mixture, centres ~ 3 * N(0, I), points =
  centre[u] + N(0, I) with u uniform over the centres.

Every generator is a pure function of its seed (numpy PCG64).
"""
from __future__ import annotations

import numpy as np

SEED = 0x686F7261  # "hora"


def rng(stream: int, seed: int = SEED) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64([seed, stream]))


def normal(n: int, d: int, sigma: float = 10.0, stream: int = 0, seed: int = SEED) -> np.ndarray:
    return (rng(stream, seed).standard_normal((n, d), dtype=np.float32) * np.float32(sigma))


def mixture_centers(n_centers: int, d: int, seed: int = SEED, spread: float = 3.0) -> np.ndarray:
    return rng(1000, seed).standard_normal((n_centers, d), dtype=np.float32) * np.float32(spread)


def mixture(n: int, d: int, n_centers: int = 1024, stream: int = 1, seed: int = SEED,
            chunk: int = 1 << 18, spread: float = 3.0) -> np.ndarray:
    """n points of the Gaussian mixture (centres ~ spread * N(0, I)),
    generated in chunks to bound memory."""
    c = mixture_centers(n_centers, d, seed, spread)
    g = rng(stream, seed)
    out = np.empty((n, d), np.float32)
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        u = g.integers(0, n_centers, hi - lo)
        out[lo:hi] = c[u]
        out[lo:hi] += g.standard_normal((hi - lo, d), dtype=np.float32)
    return out


def mixture_device(n: int, d: int, n_centers: int = 1024, stream: int = 1, seed: int = SEED,
                   spread: float = 3.0, device: str = "cuda", chunk: int = 1 << 20):
    """The same mixture law drawn by torch on the device (for index sizes
    too large to draw on the host quickly).  Seeded, but not the numbers
    mixture() draws: centres come from stream 1000 of the seed, points from
    `stream`, so calls with different streams share the centres."""
    import torch
    gc = torch.Generator(device=device)
    gc.manual_seed((seed * 1_000_003 + 1000) & 0x7FFFFFFFFFFFFFFF)
    c = torch.randn((n_centers, d), generator=gc, device=device) * spread
    g = torch.Generator(device=device)
    g.manual_seed((seed * 1_000_003 + stream) & 0x7FFFFFFFFFFFFFFF)
    out = torch.empty((n, d), dtype=torch.float32, device=device)
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        u = torch.randint(0, n_centers, (hi - lo,), generator=g, device=device)
        out[lo:hi] = c[u] + torch.randn((hi - lo, d), generator=g, device=device)
    return out
