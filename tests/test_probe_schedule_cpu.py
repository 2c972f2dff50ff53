"""The probed schedule's correctness argument, on a host model of its keys.

Keys are (distance, row) pairs compared lexicographically, as the scan's
64-bit keys are.  The probed pass keeps every row whose distance is at or
below the query's starting threshold (the scan's key test with the row part
of the threshold at its maximum); a query that kept at least R rows takes
the R best of them, any other query is answered by the chunked schedule.
Overflow (more kept rows than the candidate capacity) keeps an arbitrary
`cap` of them, and the rescans run against the R-th key of the list so far.
The model plants thresholds that are too tight, thresholds sitting exactly
on a run of tied distances, and overflow, and checks that the answer is
always the exact R-best set."""
import numpy as np


def r_best(d, R):
    order = np.lexsort((np.arange(d.size), d))
    return [(float(d[i]), int(i)) for i in order[:R]]


def chunked(d, R, c0=64, grow=1.5):
    best = sorted((float(d[i]), i) for i in range(min(c0, d.size)))[:R]
    done = min(c0, d.size)
    while done < d.size:
        c = min(d.size - done, max(int(done * grow), 32))
        thr = best[R - 1] if len(best) >= R else (np.inf, 2**32)
        cand = [(float(d[i]), i) for i in range(done, done + c) if (float(d[i]), i) < thr]
        best = sorted(set(best) | set(cand))[:R]
        done += c
    return best


def probed(d, R, tau0, cap, rng):
    kept = [(float(d[i]), i) for i in range(d.size) if d[i] <= tau0]
    if len(kept) < R:
        return chunked(d, R), "fallback"
    rounds = 0
    if len(kept) > cap:  # overflow: an arbitrary cap of them was stored
        stored = [kept[j] for j in rng.choice(len(kept), cap, replace=False)]
        best = sorted(stored)[:R]
        while True:
            rounds += 1
            thr = best[R - 1]
            hits = [(float(d[i]), i) for i in range(d.size) if (float(d[i]), i) < thr]
            new = sorted(set(best) | set(hits))
            if len(hits) <= cap:
                return new[:R], "rescans"
            stored = [hits[j] for j in rng.choice(len(hits), cap, replace=False)]
            best = sorted(set(best) | set(stored))[:R]
            assert rounds < 64
    return sorted(kept)[:R], "probed"


def test_certificate_fallback_and_overflow():
    rng = np.random.default_rng(11)
    R, n = 20, 3000
    for trial in range(40):
        d = rng.integers(0, 400, n).astype(np.float32)  # many ties
        exact = r_best(d, R)
        kth = exact[R - 1][0]
        sub = rng.choice(n, 200, replace=False)
        probe_kth = float(np.sort(d[sub])[R - 1])  # R-th of a subset: >= kth
        cases = {
            "subset": probe_kth,
            "on the tie run": kth,
            "too tight": kth - 1.0,
            "nothing": -np.inf,
        }
        for name, tau0 in cases.items():
            got, how = probed(d, R, tau0, cap=10_000, rng=rng)
            assert got == exact, (trial, name)
            if name in ("too tight", "nothing"):
                assert how == "fallback"
            else:
                assert how == "probed"
        # loose threshold and a small capacity: the rescans converge
        got, how = probed(d, R, float(np.max(d)), cap=64, rng=rng)
        assert got == exact and how == "rescans"
