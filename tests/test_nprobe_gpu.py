"""Learned nprobe: the MLP kernels against the oracle's gradients, label
generation, training on the GPU, and what the trained model gains over
fixed-nprobe search at equal recall."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradients_match_oracle(hora, oracle, gpu):
    import ctypes as C
    rng = np.random.default_rng(0)
    f, h1, h2 = 40, 64, 64
    npar = h1 * f + h1 + h2 * h1 + h2 + h2 + 1
    p = (rng.standard_normal(npar) * 0.2).astype(np.float32)
    x = rng.standard_normal((300, f)).astype(np.float32)
    y = rng.standard_normal(300).astype(np.float32)
    lib = hora.lib()
    out = np.empty(300, np.float32)
    assert lib.hora_mlp_forward(C.c_void_p(p.ctypes.data), f, h1, h2, C.c_void_p(x.ctypes.data), 300,
                                C.c_void_p(out.ctypes.data)) == 0
    np.testing.assert_allclose(out, oracle.mlp_forward(p, x, f, h1, h2), rtol=1e-4, atol=1e-4)
    g = np.empty(npar, np.float32)
    loss = C.c_float()
    assert lib.hora_mlp_loss_grad(C.c_void_p(p.ctypes.data), f, h1, h2, C.c_void_p(x.ctypes.data),
                                  C.c_void_p(y.ctypes.data), 300, C.c_float(2.5), C.byref(loss),
                                  C.c_void_p(g.ctypes.data)) == 0
    ref_loss, ref_g = oracle.mlp_loss_grad(p, x, y, f, h1, h2, alpha=2.5)
    assert abs(loss.value - ref_loss) <= 1e-4 * abs(ref_loss)
    # FP32 sums vs the FP64 oracle
    np.testing.assert_allclose(g, ref_g, rtol=2e-3, atol=2e-5 * np.abs(ref_g).max())


def _ivf(hora, synth, n=200_000, d=64, lists=256):
    # overlapping clusters: neighbours spread over several lists, so the
    # nprobe a query needs varies (well-separated clusters need one list)
    X = synth.mixture(n, d, 512, stream=51, spread=1.2)
    p = hora.IVFPQParams(n_sub=16, sub_bits=8, n_kmeans_center=lists, search_n_center=8,
                         train_epoch=6)
    ix = hora.IVFPQIndex(d, p)
    ix.madd(X, None)
    ix.build(hora.Metric.Euclidean)
    ix.set_option(hora.Option.IVF_RERANK, 100)
    return ix, X


def test_learned_nprobe_trains_and_gains(hora, oracle, gpu):
    from hora_gb300 import synth
    ix, X = _ivf(hora, synth)
    train = synth.mixture(20_000, 64, 512, stream=52, spread=1.2)
    held = synth.mixture(2_000, 64, 512, stream=53, spread=1.2)
    stats = ix.train_nprobe(train, max_nprobe=64, recall_target=0.9, epochs=20)
    assert np.isfinite(stats[0]) and stats[2] <= 6.0
    # exact neighbours of the held-out queries
    bfi = hora.BruteForceIndex(64)
    bfi.madd(X, None)
    bfi.build(hora.Metric.Euclidean)
    exact, _ = bfi.search_batch(held, 10)

    def rec(ids):
        return np.mean([len(set(a.tolist()) & set(b.tolist())) / 10 for a, b in zip(ids, exact)])

    fixed = {}
    for npb in (1, 2, 4, 8, 16, 32, 64):
        ids, _ = ix.search_batch(held, 10, nprobe=npb)
        fixed[npb] = rec(ids)
    ix.set_option(hora.Option.LEARNED_NPROBE, 1)
    ix.set_option(hora.Option.NPROBE_MARGIN, 1.0)
    ids, d = ix.search_batch(held, 10)
    r_learned = rec(ids)
    pred = ix.predict_nprobe(held)
    mean_probes = float(np.maximum(pred, 4).mean())
    # the gain: fewer probes than the smallest fixed nprobe reaching the same
    # recall, or more recall than fixed search at the same average probes
    need = min([p for p, r in fixed.items() if r >= r_learned - 1e-9] or [64])
    grid = sorted(fixed)
    m = min(max(mean_probes, 1.0), 64.0)
    lo = max(p for p in grid if p <= m)
    hi = min(p for p in grid if p >= m)
    w = 0.0 if hi == lo else (np.log2(m) - np.log2(lo)) / (np.log2(hi) - np.log2(lo))
    fixed_at_same_cost = fixed[lo] + w * (fixed[hi] - fixed[lo])
    print("fixed", fixed, "learned", r_learned, "mean probes", mean_probes, "fixed needs", need,
          "fixed at the same cost", fixed_at_same_cost)
    assert r_learned >= 0.95
    assert mean_probes < need or r_learned > fixed_at_same_cost + 0.002, \
        (mean_probes, need, fixed, r_learned)
    # features are finite and the model's nprobe respects the clamp
    F = ix.nprobe_features(held[:64])
    assert F.shape == (64, 40) and np.isfinite(F).all()
    assert pred.min() >= 1 and pred.max() <= 64
