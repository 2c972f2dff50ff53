"""The margin of the BF16 starting-threshold probe, checked on the host.

The probe scores a query against pivot-cluster rows with the scan's
arithmetic (BF16 operands, exact products, f32 sums, the folded norm) but in
its own summation order: one f32 FMA per dimension in dimension order, then
-|x|^2/2 in one add.  The tensor cores add the same exact products in K
blocks of 16 (order and internal width unspecified) and the norm as three
BF16 parts.  The threshold adds 1e-4 (|q|^2 + max |x|^2) on top of the R-th
probe distance; this test measures the difference between the two orders
(sequential vs. blocked pairwise sums, and a truncating accumulator) against
that margin on mixture data, on data far from the origin, and on adversarial
signs.  A margin that is too small only costs speed (the pass certifies
itself per query); this pins that it is ample for the data the bench uses."""
import numpy as np


def bf16(x):
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def seq_sum(prods, fold):
    acc = np.zeros(prods.shape[0], np.float32)
    for k in range(prods.shape[1]):
        acc = (acc + prods[:, k]).astype(np.float32)
    return (acc + fold).astype(np.float32)


def to_f32(v64, truncate):
    r = v64.astype(np.float32)
    if truncate:  # round toward zero instead of to nearest
        over = np.abs(r.astype(np.float64)) > np.abs(v64)
        r[over] = np.nextafter(r[over], np.float32(0))
    return r


def blocked_sum(prods, parts, truncate=False):
    """K blocks of 16: pairwise tree inside a block, blocks added in order,
    then the three norm parts as one more block; every add rounded to f32
    (to nearest, or toward zero)."""
    acc = np.zeros(prods.shape[0], np.float32)
    blocks = [prods[:, i:i + 16] for i in range(0, prods.shape[1], 16)] + [parts]
    for blk in blocks:
        v = blk.astype(np.float32)
        while v.shape[1] > 1:
            if v.shape[1] % 2:
                v = np.concatenate([v, np.zeros((v.shape[0], 1), np.float32)], axis=1)
            v = to_f32(v[:, 0::2].astype(np.float64) + v[:, 1::2], truncate)
        acc = to_f32(acc.astype(np.float64) + v[:, 0], truncate)
    return acc


def fold_parts(xsq64):
    v = (-0.5 * xsq64).astype(np.float32)
    h1 = bf16(v)
    r1 = (v - h1).astype(np.float32)
    h2 = bf16(r1)
    r2 = (r1 - h2).astype(np.float32)
    h3 = bf16(r2)
    return v, np.stack([h1, h2, h3], axis=1)


def worst_ratio(q, X):
    qb, xb = bf16(q), bf16(X)
    prods = (qb[None, :].astype(np.float64) * xb.astype(np.float64)).astype(np.float32)
    assert np.array_equal(prods.astype(np.float64), qb[None, :].astype(np.float64) * xb.astype(np.float64))
    xsq64 = (X.astype(np.float64) ** 2).sum(1)
    v, parts = fold_parts(xsq64)
    qa = np.float32((q.astype(np.float64) ** 2).sum())
    d_seq = (qa - 2 * seq_sum(prods, v)).astype(np.float32)
    margin = 1e-4 * (float(qa) + float(xsq64.max()))
    worst = 0.0
    for truncate in (False, True):
        d_blk = (qa - 2 * blocked_sum(prods, parts, truncate)).astype(np.float32)
        worst = max(worst, float(np.max(np.abs(d_seq.astype(np.float64) - d_blk))) / margin)
    return worst


def test_probe_margin_covers_summation_order():
    rng = np.random.default_rng(0)
    cen = rng.standard_normal((64, 128)).astype(np.float32) * 3
    X = (cen[rng.integers(0, 64, 4000)] + rng.standard_normal((4000, 128))).astype(np.float32)
    q = (cen[3] + rng.standard_normal(128)).astype(np.float32)
    assert worst_ratio(q, X) < 0.05
    # far from the origin: large norms, small distances
    off = np.float32(50.0)
    assert worst_ratio(q + off, X + off) < 0.05
    # alternating signs: products cancel, the sum is much smaller than its terms
    s = np.where(np.arange(128) % 2, 1.0, -1.0).astype(np.float32)
    Xs = (np.abs(X) + 1.0) * s
    assert worst_ratio((np.abs(q) + 1.0) * s, Xs[:, ::-1].copy()) < 0.05


def _descent(v, R, skip, start_bit, a0):
    a = a0
    for b in range(start_bit, skip - 1, -1):
        tt = a | (1 << b)
        if int((v < tt).sum()) < R:
            a = tt
    return a | ((1 << skip) - 1)


def test_threshold_descent_starts_below_the_common_bits():
    """probe_select_kernel takes a query's R-th smallest probe key (ordered
    32-bit encoding, rounded up below bit 12) by a bitwise descent.  It
    starts below the highest bit in which the members' keys differ, with
    their common higher bits as the start: a descent through those bits
    would set exactly the ones the keys share (a set bit leaves no key below
    it, a clear one all L >= R).  The shortcut must give the full descent's
    value for every key set: random words, float-like distances, ties, one
    distinct key, and keys differing only below the rounding bit."""
    rng = np.random.default_rng(11)
    skip = 12
    for it in range(4000):
        L = int(rng.integers(1, 1025))
        R = int(rng.integers(1, L + 1))
        kind = it % 5
        if kind == 0:
            v = rng.integers(0, 2**32, L, dtype=np.uint64)
        elif kind == 1:
            v = rng.uniform(100, 300, L).astype(np.float32).view(np.uint32).astype(np.uint64)
        elif kind == 2:
            v = np.full(L, int(rng.integers(0, 2**32)), dtype=np.uint64)
        elif kind == 3:
            v = (int(rng.integers(0, 2**31)) + rng.integers(0, 5000, L)).astype(np.uint64)
        else:
            v = (int(rng.integers(0, 2**20)) * 4096 + rng.integers(0, 4096, L)).astype(np.uint64)
        lo, hi = int(v.min()), int(v.max())
        top = (lo ^ hi).bit_length() - 1
        a0 = lo if top < 0 else (0 if top >= 31 else lo & ~((2 << top) - 1) & 0xFFFFFFFF)
        assert _descent(v, R, skip, top, a0) == _descent(v, R, skip, 31, 0), (it, L, R)
