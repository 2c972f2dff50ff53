"""The per-row bound of the certified exact Euclidean search, checked on the
host.

The BF16 scan gives a row x the value s = fma(-2, acc, f32(|q|^2)) with acc
the FP32 accumulation of the exact products of the BF16-rounded query and
row plus the row's -|x|^2/2 in three BF16 parts.  The reference's distance
r is the sequential f32 sum of (q_t - x_t)^2.  The window before the exact
rescoring (exact_tc_window_kernel) relies on |s - r| <= e_r, e_r built from
the query's |bf16(q)|, |q - bf16(q)|, |q|^2 and the row's own |x|^2 and
|x - bf16(x)|.  This test evaluates e_r as the kernel does (f32, widened by
2^-8) and checks the inequality for every (query, row) pair of mixture data,
data far from the origin and near-duplicate rows, with the accumulation done
in two orders (sequential, and blocks of 16 added pairwise) since the tensor
core's internal order is not specified."""
import numpy as np


def bf16(x):
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def ref_l2(q, X):
    acc = np.zeros(X.shape[0], np.float32)
    for t in range(X.shape[1]):
        d = (q[t] - X[:, t]).astype(np.float32)
        acc = (acc + (d * d).astype(np.float32)).astype(np.float32)
    return acc


def scan_value(q, X, blocked):
    qb, xb = bf16(q), bf16(X)
    prods = (xb.astype(np.float64) * qb.astype(np.float64)).astype(np.float32)  # exact in f32
    v = (-0.5 * np.einsum("ij,ij->i", X.astype(np.float64), X.astype(np.float64))).astype(np.float32)
    h1 = bf16(v)
    r1 = (v - h1).astype(np.float32)
    h2 = bf16(r1)
    h3 = bf16((r1 - h2).astype(np.float32))
    parts = np.concatenate([prods, np.stack([h1, h2, h3], 1)], axis=1)
    if blocked:
        acc = np.zeros(X.shape[0], np.float32)
        for b0 in range(0, parts.shape[1], 16):
            blk = parts[:, b0:b0 + 16]
            while blk.shape[1] > 1:
                if blk.shape[1] % 2:
                    blk = np.concatenate([blk, np.zeros((blk.shape[0], 1), np.float32)], axis=1)
                blk = (blk[:, 0::2] + blk[:, 1::2]).astype(np.float32)
            acc = (acc + blk[:, 0]).astype(np.float32)
    else:
        acc = np.zeros(X.shape[0], np.float32)
        for t in range(parts.shape[1]):
            acc = (acc + parts[:, t]).astype(np.float32)
    qsq = np.float32(np.dot(q.astype(np.float64), q.astype(np.float64)))
    return (np.float64(qsq) - 2.0 * acc.astype(np.float64)).astype(np.float32)  # one rounding, as fmaf


def row_bound(q, X, Dp):
    f = np.float32
    qd = q.astype(np.float64)
    qbn = np.sqrt(np.sum(bf16(q).astype(np.float64) ** 2)) * (1 + 2.0 ** -40)
    dqn = np.sqrt(np.sum((qd - bf16(q)) ** 2)) * (1 + 2.0 ** -40)
    qsq64 = np.dot(qd, qd)
    qb, dq = f(qbn), f(dqn)
    qsq, qn = f(qsq64 * (1 + 2.0 ** -40)), f(np.sqrt(qsq64) * (1 + 2.0 ** -40))
    xsq = np.einsum("ij,ij->i", X.astype(np.float64), X.astype(np.float64)).astype(np.float32)
    dx = np.sqrt(np.sum((X.astype(np.float64) - bf16(X)) ** 2, axis=1)).astype(np.float32)
    dx = np.nextafter(dx, np.float32(np.inf))
    xs = (xsq * f(1 + 2.0 ** -22)).astype(np.float32)
    xn = (np.sqrt(xs) * f(1 + 2.0 ** -22)).astype(np.float32)
    xb = (xn * f(1 + 2.0 ** -8) + dx).astype(np.float32)
    A = qb * dx + dq * xn
    B = f((Dp + 16) * 2.0 ** -22) * (qb * xb + f(0.5) * xs)
    C = f(2.0 ** -22) * (qsq + f(2) * qb * xb + xs)
    E = f((X.shape[1] + 4) * 2.0 ** -23) * (qn + xn) * (qn + xn)
    return ((f(2) * A + f(2) * B + C + E) * f(1 + 2.0 ** -8)).astype(np.float32)


def check(q, X):
    Dp = ((X.shape[1] + 63) // 64) * 64
    r = ref_l2(q, X).astype(np.float64)
    e = row_bound(q, X, Dp).astype(np.float64)
    for blocked in (False, True):
        s = scan_value(q, X, blocked).astype(np.float64)
        gap = np.abs(s - r)
        assert (gap <= e).all(), (blocked, float((gap / e).max()))
        # the bound is not vacuous: within a few hundred times the gap seen
        assert np.median(e) < 1e3 * max(np.median(gap), 1e-6) + 1.0


def test_row_bound_mixture():
    rng = np.random.default_rng(5)
    cen = rng.standard_normal((32, 128)).astype(np.float32) * 3
    X = (cen[rng.integers(0, 32, 3000)] + rng.standard_normal((3000, 128))).astype(np.float32)
    for i in range(6):
        q = (cen[i] + rng.standard_normal(128)).astype(np.float32)
        check(q, X)


def test_row_bound_far_from_origin_and_near_duplicates():
    rng = np.random.default_rng(6)
    off = np.float32(100.0)
    X = (rng.standard_normal((2000, 96)) + off).astype(np.float32)
    q = X[3] + np.float32(1e-3) * rng.standard_normal(96).astype(np.float32)
    X[10:40] = X[3] + np.float32(1e-4) * rng.standard_normal((30, 96)).astype(np.float32)
    check(q.astype(np.float32), X)
    # mixed scales: rows of very different norms against one query
    Y = (rng.standard_normal((2000, 64)) * rng.uniform(0.01, 50, (2000, 1))).astype(np.float32)
    check(rng.standard_normal(64).astype(np.float32) * 5, Y)
