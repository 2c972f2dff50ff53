// nprobe_mlp.cu — learned per-query nprobe for IVF-PQ (no reference
// counterpart; the reference always probes search_n_center lists,
// src/index/pq_idx.rs:424).
//
// Search with the model: probe the p1 nearest lists (p1 = HORA_OPT_NPROBE_
// PHASE1, 0..64; 4 as the configuration states it, 0 or 1 when the probes
// themselves are the cost to save), read 40 features (the 32 smallest coarse
// distances and 8 summaries of the running top-10 after the p1 probes, all
// relative to the nearest coarse distance; with p1 = 0 the top-10 summaries
// fall back to coarse distances), predict log2(nprobe) with an MLP
// 40 -> 64 -> 64 -> 1 (ReLU, FP32 weights), probe the remaining lists of
// each query, merge, rerank.  Fixed-nprobe search stays the fallback (option
// off, or no model).
//
// Training (hora_ivfpq_train_nprobe): labels come from the method itself —
// for each training query the smallest nprobe in 1, 2, 4, ... max whose
// top-10 reaches the recall target against exact brute force (with k = 10 a
// per-query recall of 0.95 means all ten; a query that no grid nprobe brings
// there takes the smallest nprobe reaching its best recall) — and the MLP is
// fitted on the GPU
// with this file's forward / backward / Adam kernels (asymmetric squared
// error: under-predicting nprobe costs recall and is weighted more).  The
// last tenth of the training queries is held out: on it the model's margin
// (added to the predicted log2 nprobe) is calibrated as the smallest that
// keeps the held-out recall@10 at or above the target, judged by the same
// exact brute force.  The same kernels serve the gradient check against the
// oracle (hora_mlp_loss_grad).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <vector>

#include "index.h"

namespace hora {

constexpr int kF = 40, kH1 = 64, kH2 = 64;
constexpr int kMlpBatch = 128;  // samples per CTA in the backward kernel

__host__ __device__ inline int64_t mlp_nparams(int64_t f, int64_t h1, int64_t h2) {
  return h1 * f + h1 + h2 * h1 + h2 + h2 + 1;
}

struct NprobeModel {
  DevBuf params, mean, inv_std;
  int f = kF, h1 = kH1, h2 = kH2;
  int pmax = 128;
  int p1 = 4;  // lists probed before the features are read
  double final_loss = 0;
  // calibration on the held-out training queries
  double margin = 0;        // added to the predicted log2 nprobe
  double target = 0;        // recall@10 the margin was calibrated for
  double cal_recall = -1;   // held-out recall@10 at that margin
  double cal_nprobe = 0;    // held-out mean nprobe at that margin
  int64_t cal_queries = 0;
};

void nprobe_model_free(NprobeModel *p) { delete p; }

// ---- MLP kernels ----------------------------------------------------------------
// Forward of one sample by one thread; weights staged in shared memory.
__global__ void mlp_forward_kernel(const float *P, int f, int h1, int h2, const float *X, int64_t n,
                                   const float *mean, const float *inv_std, float *out) {
  extern __shared__ float sp[];
  const int np = (int)mlp_nparams(f, h1, h2);
  for (int i = threadIdx.x; i < np; i += blockDim.x) sp[i] = P[i];
  __syncthreads();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *W1 = sp, *b1 = W1 + h1 * f, *W2 = b1 + h1, *b2 = W2 + h2 * h1, *W3 = b2 + h2,
              *b3 = W3 + h2;
  float x[64], a1[64];
  for (int t = 0; t < f; ++t) {
    float v = X[i * f + t];
    x[t] = mean ? (v - mean[t]) * inv_std[t] : v;
  }
  for (int u = 0; u < h1; ++u) {
    float s = b1[u];
    for (int t = 0; t < f; ++t) s = fmaf(W1[u * f + t], x[t], s);
    a1[u] = fmaxf(s, 0.0f);
  }
  float o = b3[0];
  for (int u = 0; u < h2; ++u) {
    float s = b2[u];
    for (int t = 0; t < h1; ++t) s = fmaf(W2[u * h1 + t], a1[t], s);
    o = fmaf(W3[u], fmaxf(s, 0.0f), o);
  }
  out[i] = o;
}

// Forward + backward of kMlpBatch samples per CTA (one thread per sample),
// per-CTA gradient sums in a fixed order (deterministic).  Loss per sample:
// w * (out - y)^2 / n_total, w = alpha where out < y.
__global__ void __launch_bounds__(kMlpBatch) mlp_fwd_bwd_kernel(
    const float *P, int f, int h1, int h2, const float *X, const float *Y, const int *idx,
    int64_t n, int64_t n_total, float alpha, float *grad_part, float *loss_part) {
  extern __shared__ float sm[];
  const int np = (int)mlp_nparams(f, h1, h2);
  float *sp = sm;                          // params
  float *sx = sp + np;                     // B x f
  float *sa1 = sx + kMlpBatch * f;         // B x h1 (activations)
  float *sa2 = sa1 + kMlpBatch * h1;       // B x h2
  float *sd1 = sa2 + kMlpBatch * h2;       // B x h1 (pre-activation grads)
  float *sd2 = sd1 + kMlpBatch * h1;       // B x h2
  float *sdo = sd2 + kMlpBatch * h2;       // B
  float *sls = sdo + kMlpBatch;            // B
  for (int i = threadIdx.x; i < np; i += blockDim.x) sp[i] = P[i];
  const float *W1 = sp, *b1 = W1 + h1 * f, *W2 = b1 + h1, *b2 = W2 + h2 * h1, *W3 = b2 + h2,
              *b3 = W3 + h2;
  const int b = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * kMlpBatch + b;
  const bool live = i < n;
  const int64_t src = live ? (idx ? idx[i] : i) : 0;
  for (int t = 0; t < f; ++t) sx[b * f + t] = live ? X[src * f + t] : 0.0f;
  __syncthreads();
  // forward
  float o = b3[0];
  for (int u = 0; u < h1; ++u) {
    float s = b1[u];
    for (int t = 0; t < f; ++t) s = fmaf(W1[u * f + t], sx[b * f + t], s);
    sa1[b * h1 + u] = fmaxf(s, 0.0f);
  }
  for (int u = 0; u < h2; ++u) {
    float s = b2[u];
    for (int t = 0; t < h1; ++t) s = fmaf(W2[u * h1 + t], sa1[b * h1 + t], s);
    float a = fmaxf(s, 0.0f);
    sa2[b * h2 + u] = a;
    o = fmaf(W3[u], a, o);
  }
  // backward of this sample
  float y = live ? Y[src] : 0.0f;
  float r = o - y;
  float w = o < y ? alpha : 1.0f;
  float dout = live ? 2.0f * w * r / (float)n_total : 0.0f;
  sdo[b] = dout;
  sls[b] = live ? w * r * r : 0.0f;
  for (int u = 0; u < h2; ++u) sd2[b * h2 + u] = sa2[b * h2 + u] > 0.0f ? dout * W3[u] : 0.0f;
  for (int t = 0; t < h1; ++t) {
    float s = 0.0f;
    for (int u = 0; u < h2; ++u) s = fmaf(sd2[b * h2 + u], W2[u * h1 + t], s);
    sd1[b * h1 + t] = sa1[b * h1 + t] > 0.0f ? s : 0.0f;
  }
  __syncthreads();
  // batch sums of the parameter gradients, one parameter per thread per pass
  float *g = grad_part + (int64_t)blockIdx.x * np;
  float *gW1 = g, *gb1 = gW1 + h1 * f, *gW2 = gb1 + h1, *gb2 = gW2 + h2 * h1, *gW3 = gb2 + h2,
        *gb3 = gW3 + h2;
  for (int e = threadIdx.x; e < h1 * f; e += blockDim.x) {
    int u = e / f, t = e % f;
    float s = 0.0f;
    for (int bb = 0; bb < kMlpBatch; ++bb) s = fmaf(sd1[bb * h1 + u], sx[bb * f + t], s);
    gW1[e] = s;
  }
  for (int u = threadIdx.x; u < h1; u += blockDim.x) {
    float s = 0.0f;
    for (int bb = 0; bb < kMlpBatch; ++bb) s += sd1[bb * h1 + u];
    gb1[u] = s;
  }
  for (int e = threadIdx.x; e < h2 * h1; e += blockDim.x) {
    int u = e / h1, t = e % h1;
    float s = 0.0f;
    for (int bb = 0; bb < kMlpBatch; ++bb) s = fmaf(sd2[bb * h2 + u], sa1[bb * h1 + t], s);
    gW2[e] = s;
  }
  for (int u = threadIdx.x; u < h2; u += blockDim.x) {
    float s = 0.0f, s3 = 0.0f;
    for (int bb = 0; bb < kMlpBatch; ++bb) {
      s += sd2[bb * h2 + u];
      s3 = fmaf(sdo[bb], sa2[bb * h2 + u], s3);
    }
    gb2[u] = s;
    gW3[u] = s3;
  }
  if (threadIdx.x == 0) {
    float s = 0.0f, l = 0.0f;
    for (int bb = 0; bb < kMlpBatch; ++bb) {
      s += sdo[bb];
      l += sls[bb];
    }
    gb3[0] = s;
    loss_part[blockIdx.x] = l;
  }
}

// Sums the per-CTA gradients (fixed order) and, if lr > 0, applies Adam.
__global__ void mlp_reduce_adam_kernel(const float *grad_part, int G, int np, float *grad_out,
                                       float *P, float *m, float *v, int step, float lr) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= np) return;
  float g = 0.0f;
  for (int c = 0; c < G; ++c) g += grad_part[(int64_t)c * np + e];
  if (grad_out) grad_out[e] = g;
  if (lr > 0.0f) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float mm = b1 * m[e] + (1 - b1) * g;
    float vv = b2 * v[e] + (1 - b2) * g * g;
    m[e] = mm;
    v[e] = vv;
    float mh = mm / (1 - powf(b1, (float)step));
    float vh = vv / (1 - powf(b2, (float)step));
    P[e] -= lr * mh / (sqrtf(vh) + eps);
  }
}

static int mlp_smem(int f, int h1, int h2) {
  return (int)(mlp_nparams(f, h1, h2) + kMlpBatch * (f + 2 * h1 + 2 * h2 + 2)) * 4;
}

// loss and gradient over n samples; optional Adam step
static int mlp_step(const float *P, int f, int h1, int h2, const float *X, const float *Y,
                    const int *idx, int64_t n, float alpha, DevBuf &gpart, DevBuf &lpart,
                    float *grad_out, float *m, float *v, int step, float lr, float *Pw,
                    cudaStream_t s) {
  const int np = (int)mlp_nparams(f, h1, h2);
  const int G = ceil_div(n, kMlpBatch);
  HORA_TRY(gpart.reserve(sizeof(float) * (size_t)G * np));
  HORA_TRY(lpart.reserve(sizeof(float) * G));
  const int smem = mlp_smem(f, h1, h2);
  HORA_SMEM_ATTR(mlp_fwd_bwd_kernel, smem);
  {
    ProfScope ps("mlp_fwd_bwd", s);
    mlp_fwd_bwd_kernel<<<G, kMlpBatch, smem, s>>>(P, f, h1, h2, X, Y, idx, n, n, alpha,
                                                   gpart.as<float>(), lpart.as<float>());
    HORA_LAUNCHED();
  }
  {
    ProfScope ps("mlp_adam", s);
    mlp_reduce_adam_kernel<<<ceil_div(np, 256), 256, 0, s>>>(gpart.as<float>(), G, np, grad_out, Pw, m, v,
                                                             step, lr);
    HORA_LAUNCHED();
  }
  return HORA_OK;
}

static int mlp_forward(const float *P, int f, int h1, int h2, const float *X, int64_t n,
                       const float *mean, const float *inv_std, float *out, cudaStream_t s) {
  if (n <= 0) return HORA_OK;
  const int smem = (int)mlp_nparams(f, h1, h2) * 4;
  ProfScope ps("mlp_forward", s);
  mlp_forward_kernel<<<ceil_div(n, 128), 128, smem, s>>>(P, f, h1, h2, X, n, mean, inv_std, out);
  HORA_LAUNCHED();
  return HORA_OK;
}

// ---- features -----------------------------------------------------------------------
// probes: nq x pw sorted coarse keys (pw >= 32); M: nq x R sorted keys after
// the first probes.  Missing entries repeat the last valid one.
__global__ void nprobe_features_kernel(const uint64_t *probes, int pw, const uint64_t *M, int R,
                                       int64_t nq, float *F) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  float d[32], t[10];
  float last = 0.0f;
  for (int i = 0; i < 32; ++i) {
    uint64_t k = i < pw ? probes[q * pw + i] : kEmptyKey;
    if (k != kEmptyKey) last = key_dist(k);
    d[i] = last;
  }
  float lt = d[31];
  for (int i = 0; i < 10; ++i) {
    uint64_t k = i < R ? M[q * R + i] : kEmptyKey;
    if (k != kEmptyKey) lt = key_dist(k);
    t[i] = lt;
  }
  const float d0 = d[0], sc = fabsf(d0) + 1e-6f;
  float *f = F + q * kF;
  f[0] = logf(sc);
  for (int i = 1; i < 32; ++i) f[i] = (d[i] - d0) / sc;
  f[32] = (t[0] - d0) / sc;
  f[33] = (t[9] - d0) / sc;
  f[34] = (t[9] - t[0]) / sc;
  f[35] = (d[4] - t[9]) / sc;
  f[36] = (d[8] - t[9]) / sc;
  f[37] = (t[4] - t[0]) / sc;
  f[38] = (d[16] - t[9]) / sc;
  f[39] = (d[31] - t[9]) / sc;
}

__global__ void predict_nprobe_kernel(const float *pred, int64_t nq, float margin, int lo, int hi,
                                      uint32_t *out) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  float e = fminf(pred[q] + margin, 20.0f);
  int p = (int)ceilf(exp2f(e) - 1e-4f);
  out[q] = (uint32_t)min(max(p, lo), hi);
}

__global__ void fill_u32_kernel(uint32_t *a, int64_t n, uint32_t v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// per query, the number of its exact top-10 rows found by the search at
// grid nprobe number gi (the labels and the margin calibration read these)
__global__ void hits_kernel(const uint64_t *res, int kr, const uint64_t *exact, int ke, int64_t nq,
                            uint8_t *hits, int gi, int ng) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  int hit = 0, tot = 0;
  for (int i = 0; i < ke; ++i) {
    uint64_t e = exact[q * ke + i];
    if (e == kEmptyKey) continue;
    ++tot;
    for (int j = 0; j < kr; ++j)
      if (res[q * kr + j] != kEmptyKey && key_row(res[q * kr + j]) == key_row(e)) {
        ++hit;
        break;
      }
  }
  hits[q * ng + gi] = (uint8_t)(tot == 0 ? ke : hit);
}

// ---- search with the model ---------------------------------------------------------------
static int learned_nprobe_per_query(hora_index *h, int64_t nq, int R, uint64_t *M, SearchWorkspace &ws,
                                    int pw, DevBuf &np_q, cudaStream_t s) {
  NprobeModel &md = *h->nprobe;
  // phase 1: the p1 nearest lists (none when p1 = 0)
  HORA_TRY(np_q.reserve(sizeof(uint32_t) * std::max<int64_t>(nq, 1)));
  const int p1 = std::min(md.p1, pw);
  HORA_CUDA_TRY(cudaMemsetAsync(M, 0xff, sizeof(uint64_t) * nq * R, s));
  if (p1 > 0) {
    fill_u32_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(np_q.as<uint32_t>(), nq, (uint32_t)p1);
    HORA_LAUNCHED();
    HORA_TRY(ivf_adc_merge(h, nq, pw, 0, np_q.as<uint32_t>(), R, M, ws, s));
  }
  // features -> MLP -> nprobe
  HORA_TRY(ws.feats.reserve(sizeof(float) * nq * kF));
  HORA_TRY(ws.pred.reserve(sizeof(float) * std::max<int64_t>(nq, 1)));
  {
    ProfScope ps("nprobe_features", s);
    nprobe_features_kernel<<<ceil_div(nq, 128), 128, 0, s>>>(ivf_probe_keys(ws), pw, M, R, nq, ws.feats.as<float>());
    HORA_LAUNCHED();
  }
  HORA_TRY(mlp_forward(md.params.as<float>(), md.f, md.h1, md.h2, ws.feats.as<float>(), nq,
                       md.mean.as<float>(), md.inv_std.as<float>(), ws.pred.as<float>(), s));
  const int hi = std::min(pw, h->nprobe_max > 0 ? h->nprobe_max : md.pmax);
  predict_nprobe_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(ws.pred.as<float>(), nq,
                                                          (float)(md.margin + h->nprobe_margin),
                                                          std::max(1, p1), std::max(hi, p1),
                                                          np_q.as<uint32_t>());
  HORA_LAUNCHED();
  return HORA_OK;
}

static int learned_width(hora_index *h) {
  const int C = (int)h->ivf.n_kmeans_center;
  int pm = h->nprobe_max > 0 ? h->nprobe_max : h->nprobe->pmax;
  return std::min(C, std::max(32, pm));
}

std::string nprobe_model_info(const hora_index *h) {
  if (!h->nprobe) return "null";
  const NprobeModel &m = *h->nprobe;
  char buf[320];
  std::snprintf(buf, sizeof(buf),
                "{\"phase1\":%d,\"pmax\":%d,\"final_loss\":%.6g,\"target\":%.6g,\"margin\":%.6g,"
                "\"heldout_queries\":%lld,\"heldout_recall\":%.6g,\"heldout_mean_nprobe\":%.6g}",
                m.p1, m.pmax, m.final_loss, m.target, m.margin, (long long)m.cal_queries, m.cal_recall,
                m.cal_nprobe);
  return buf;
}

int ivf_search_learned(hora_index *h, int64_t nq, int k, SearchWorkspace &ws, uint64_t *d_best,
                       cudaStream_t s) {
  const int pw = learned_width(h);
  const int R = ivf_rerank_width(h, k);
  HORA_TRY(ivf_probe(h, nq, pw, ws, s));
  uint64_t *M = ivf_merge_buffer(ws, nq, R, d_best, k);
  if (!M) return fail(HORA_EOOM, "IVF-PQ: merge buffer");
  DevBuf &npq = ws.npq;
  HORA_TRY(learned_nprobe_per_query(h, nq, R, M, ws, pw, npq, s));
  // phase 2: the remaining lists of each query
  HORA_TRY(ivf_adc_merge(h, nq, pw, h->nprobe->p1, npq.as<uint32_t>(), R, M, ws, s));
  return ivf_finalize(h, nq, k, R, M, ws, d_best, s);
}

}  // namespace hora

using namespace hora;

extern "C" {

int hora_mlp_forward(const float *params, uint64_t f, uint64_t h1, uint64_t h2, const float *x,
                     uint64_t n, float *out) {
  if (!params || !x || !out) return fail(HORA_EINVAL, "null buffer");
  if (f > 64 || h1 > 64 || h2 > 64 || f == 0 || h1 == 0 || h2 == 0)
    return fail(HORA_ECAP, "MLP widths must be in [1, 64]");
  const int64_t np = mlp_nparams(f, h1, h2);
  DevBuf P, X, O;
  HORA_TRY(P.reserve(4 * np));
  HORA_TRY(X.reserve(4 * std::max<uint64_t>(n * f, 1)));
  HORA_TRY(O.reserve(4 * std::max<uint64_t>(n, 1)));
  HORA_CUDA_TRY(cudaMemcpy(P.ptr, params, 4 * np, cudaMemcpyHostToDevice));
  HORA_CUDA_TRY(cudaMemcpy(X.ptr, x, 4 * n * f, cudaMemcpyHostToDevice));
  HORA_TRY(mlp_forward(P.as<float>(), (int)f, (int)h1, (int)h2, X.as<float>(), (int64_t)n, nullptr,
                       nullptr, O.as<float>(), 0));
  HORA_CUDA_TRY(cudaMemcpy(out, O.ptr, 4 * n, cudaMemcpyDeviceToHost));
  return HORA_OK;
}

int hora_mlp_loss_grad(const float *params, uint64_t f, uint64_t h1, uint64_t h2, const float *x,
                       const float *y, uint64_t n, float alpha, float *loss_out, float *grad_out) {
  if (!params || !x || !y || !grad_out) return fail(HORA_EINVAL, "null buffer");
  if (f > 64 || h1 > 64 || h2 > 64 || f == 0 || h1 == 0 || h2 == 0 || n == 0)
    return fail(HORA_ECAP, "MLP widths must be in [1, 64], n > 0");
  const int64_t np = mlp_nparams(f, h1, h2);
  DevBuf P, X, Y, G, gp, lp;
  HORA_TRY(P.reserve(4 * np));
  HORA_TRY(X.reserve(4 * n * f));
  HORA_TRY(Y.reserve(4 * n));
  HORA_TRY(G.reserve(4 * np));
  HORA_CUDA_TRY(cudaMemcpy(P.ptr, params, 4 * np, cudaMemcpyHostToDevice));
  HORA_CUDA_TRY(cudaMemcpy(X.ptr, x, 4 * n * f, cudaMemcpyHostToDevice));
  HORA_CUDA_TRY(cudaMemcpy(Y.ptr, y, 4 * n, cudaMemcpyHostToDevice));
  HORA_TRY(mlp_step(P.as<float>(), (int)f, (int)h1, (int)h2, X.as<float>(), Y.as<float>(), nullptr,
                    (int64_t)n, alpha, gp, lp, G.as<float>(), nullptr, nullptr, 0, 0.0f, nullptr, 0));
  HORA_CUDA_TRY(cudaMemcpy(grad_out, G.ptr, 4 * np, cudaMemcpyDeviceToHost));
  if (loss_out) {
    const int Gc = ceil_div(n, kMlpBatch);
    std::vector<float> l(Gc);
    HORA_CUDA_TRY(cudaMemcpy(l.data(), lp.ptr, 4 * Gc, cudaMemcpyDeviceToHost));
    double s = 0;
    for (float v : l) s += v;
    *loss_out = (float)(s / (double)n);
  }
  return HORA_OK;
}

int hora_ivfpq_nprobe_features(hora_index *h, const float *queries, uint64_t nq, float *features_out) {
  if (!h || !queries || !features_out) return fail(HORA_EINVAL, "null argument");
  if (h->kind != HORA_INDEX_IVFPQ || !h->ivfs) return fail(HORA_ENOTBUILT, "IVF-PQ index not built");
  if (nq == 0) return HORA_OK;
  std::lock_guard<std::mutex> g(h->mu);
  cudaStream_t s = h->stream;
  SearchWorkspace &ws = h->ws;
  HORA_TRY(stage_queries(h, queries, (int64_t)nq, ws, s));
  const int C = (int)h->ivf.n_kmeans_center;
  const int pw = std::min(C, 32);
  const int R = 10;
  HORA_TRY(ivf_probe(h, (int64_t)nq, pw, ws, s));
  DevBuf M, npq, F;
  HORA_TRY(M.reserve(8 * nq * R));
  HORA_TRY(npq.reserve(4 * nq));
  HORA_TRY(F.reserve(4 * nq * kF));
  fill_u32_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(npq.as<uint32_t>(), nq,
                                                    (uint32_t)std::min(h->nprobe ? h->nprobe->p1 : h->nprobe_phase1, pw));
  HORA_LAUNCHED();
  HORA_CUDA_TRY(cudaMemsetAsync(M.ptr, 0xff, 8 * nq * R, s));
  HORA_TRY(ivf_adc_merge(h, (int64_t)nq, pw, 0, npq.as<uint32_t>(), R, M.as<uint64_t>(), ws, s));
  nprobe_features_kernel<<<ceil_div(nq, 128), 128, 0, s>>>(ivf_probe_keys(ws), pw, M.as<uint64_t>(), R,
                                                           (int64_t)nq, F.as<float>());
  HORA_LAUNCHED();
  HORA_CUDA_TRY(cudaMemcpyAsync(features_out, F.ptr, 4 * nq * kF, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  return HORA_OK;
}

int hora_ivfpq_predict_nprobe(hora_index *h, const float *queries, uint64_t nq, uint32_t *out) {
  if (!h || !queries || !out) return fail(HORA_EINVAL, "null argument");
  if (h->kind != HORA_INDEX_IVFPQ || !h->ivfs) return fail(HORA_ENOTBUILT, "IVF-PQ index not built");
  if (!h->nprobe) return fail(HORA_ENOTBUILT, "no nprobe model: call hora_ivfpq_train_nprobe");
  if (nq == 0) return HORA_OK;
  std::lock_guard<std::mutex> g(h->mu);
  cudaStream_t s = h->stream;
  SearchWorkspace &ws = h->ws;
  HORA_TRY(stage_queries(h, queries, (int64_t)nq, ws, s));
  const int pw = learned_width(h);
  const int R = 10;
  HORA_TRY(ivf_probe(h, (int64_t)nq, pw, ws, s));
  DevBuf M, npq;
  HORA_TRY(M.reserve(8 * nq * R));
  HORA_TRY(learned_nprobe_per_query(h, (int64_t)nq, R, M.as<uint64_t>(), ws, pw, npq, s));
  HORA_CUDA_TRY(cudaMemcpyAsync(out, npq.ptr, 4 * nq, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  return HORA_OK;
}

int hora_ivfpq_train_nprobe(hora_index *h, const float *train_queries, uint64_t n_train,
                            uint64_t max_nprobe, double recall_target, uint64_t epochs,
                            double *stats_out) {
  if (!h || !train_queries) return fail(HORA_EINVAL, "null argument");
  if (h->kind != HORA_INDEX_IVFPQ || !h->ivfs) return fail(HORA_ENOTBUILT, "IVF-PQ index not built");
  if (n_train < kMlpBatch) return fail(HORA_EINVAL, "need at least 128 training queries");
  if (!(recall_target > 0.0 && recall_target <= 1.0)) return fail(HORA_EINVAL, "recall target must be in (0, 1]");
  HORA_TRY(check_not_foreign(train_queries, "train_queries"));
  std::lock_guard<std::mutex> g(h->mu);
  cudaStream_t s = h->stream;
  SearchWorkspace &ws = h->ws;
  const int C = (int)h->ivf.n_kmeans_center;
  const int pm = (int)std::min<uint64_t>(std::max<uint64_t>(max_nprobe, 1), (uint64_t)C);
  const int pw = std::min(C, std::max(32, pm));
  const int kk = 10;
  const int p1 = std::min(h->nprobe_phase1, pw);
  const int R = ivf_rerank_width(h, kk);
  std::vector<int> grid;
  for (int p = 1; p < pm; p *= 2) grid.push_back(p);
  grid.push_back(pm);
  const int ng = (int)grid.size();
  const int64_t N = (int64_t)n_train;
  // the last tenth is held out for the margin calibration
  const int64_t n_cal = N >= 2048 ? N / 10 : 0;
  const int64_t N_fit = N - n_cal;
  DevBuf feats, labels, hits, exact, res, M, npq;
  HORA_TRY(feats.reserve(4 * N * kF));
  HORA_TRY(labels.reserve(4 * N));
  HORA_TRY(hits.reserve((size_t)N * ng));
  const int64_t chunk = 8192;
  HORA_TRY(exact.reserve(8 * chunk * kk));
  HORA_TRY(res.reserve(8 * chunk * kk));
  HORA_TRY(M.reserve(8 * chunk * std::max(R, kk)));
  HORA_TRY(npq.reserve(4 * chunk));
  const int saved_learned = h->learned_nprobe;
  h->learned_nprobe = 0;
  BaseView bv = base_view(h);
  if (h->metric == M_COS) HORA_TRY(ensure_norms(h, s));
  bv.xnorm = h->xnorm.as<float>();
  for (int64_t lo = 0; lo < N; lo += chunk) {
    const int64_t nq = std::min(chunk, N - lo);
    HORA_TRY(stage_queries(h, train_queries + lo * h->dim, nq, ws, s));
    // exact top-10 (the judge of the labels)
    int retries = 0;
    HORA_TRY(bf_topk_exact(bv, h->metric, ws.q.as<float>(), ws.qnorm.as<float>(), nq, kk, h->cand_cap,
                           ws, exact.as<uint64_t>(), s, &retries));
    // hits at every grid nprobe (the labels are derived from them below)
    for (int gi = 0; gi < ng; ++gi) {
      HORA_TRY(ivf_search_keys(h, nq, kk, grid[gi], nullptr, ws, res.as<uint64_t>(), s));
      hits_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(res.as<uint64_t>(), kk, exact.as<uint64_t>(), kk, nq,
                                                    hits.as<uint8_t>() + lo * ng, gi, ng);
      HORA_LAUNCHED();
    }
    // features after the first p1 probes
    HORA_TRY(ivf_probe(h, nq, pw, ws, s));
    HORA_CUDA_TRY(cudaMemsetAsync(M.ptr, 0xff, 8 * nq * R, s));
    if (p1 > 0) {
      fill_u32_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(npq.as<uint32_t>(), nq, (uint32_t)p1);
      HORA_LAUNCHED();
      HORA_TRY(ivf_adc_merge(h, nq, pw, 0, npq.as<uint32_t>(), R, M.as<uint64_t>(), ws, s));
    }
    nprobe_features_kernel<<<ceil_div(nq, 128), 128, 0, s>>>(ivf_probe_keys(ws), pw, M.as<uint64_t>(), R, nq,
                                                             feats.as<float>() + lo * kF);
    HORA_LAUNCHED();
  }
  h->learned_nprobe = saved_learned;
  // feature standardisation over the fitted queries (statistics on the
  // host, applied in the forward)
  std::vector<float> hf(N * kF), hl(N);
  std::vector<uint8_t> hh((size_t)N * ng);
  HORA_CUDA_TRY(cudaMemcpyAsync(hf.data(), feats.ptr, 4 * N * kF, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaMemcpyAsync(hh.data(), hits.ptr, (size_t)N * ng, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  // label: log2 of the smallest grid nprobe whose top-10 reaches the target
  // (ceil(target x 10) of the exact ten: all ten for 0.95); a query whose
  // best recall over the whole grid stays below that (its neighbours are
  // lost to PQ error, not to unprobed lists) is labelled with the smallest
  // nprobe reaching that best recall: more lists would not help it
  const int need = (int)std::ceil(recall_target * kk - 1e-6);
  for (int64_t i = 0; i < N; ++i) {
    const uint8_t *hq = hh.data() + (size_t)i * ng;
    int best = 0;
    for (int gi = 0; gi < ng; ++gi) best = std::max(best, (int)hq[gi]);
    const int reach = std::min(need, best);
    int gi = 0;
    while (gi + 1 < ng && hq[gi] < reach) ++gi;
    hl[i] = std::log2((float)grid[gi]);
  }
  HORA_CUDA_TRY(cudaMemcpyAsync(labels.ptr, hl.data(), 4 * N, cudaMemcpyHostToDevice, s));
  std::vector<float> mean(kF, 0.0f), inv(kF, 1.0f);
  for (int t = 0; t < kF; ++t) {
    double m = 0, v = 0;
    for (int64_t i = 0; i < N_fit; ++i) m += hf[i * kF + t];
    m /= N_fit;
    for (int64_t i = 0; i < N_fit; ++i) v += (hf[i * kF + t] - m) * (hf[i * kF + t] - m);
    v /= N_fit;
    mean[t] = (float)m;
    inv[t] = (float)(1.0 / std::sqrt(v + 1e-6));
  }
  // standardised copy (all queries: the held-out ones are predicted from it)
  for (int64_t i = 0; i < N; ++i)
    for (int t = 0; t < kF; ++t) hf[i * kF + t] = (hf[i * kF + t] - mean[t]) * inv[t];
  HORA_CUDA_TRY(cudaMemcpyAsync(feats.ptr, hf.data(), 4 * N * kF, cudaMemcpyHostToDevice, s));
  // parameters: He-uniform init from the handle's seed
  std::unique_ptr<NprobeModel, NprobeDeleter> md(new NprobeModel());
  const int np = (int)mlp_nparams(kF, kH1, kH2);
  std::vector<float> P(np, 0.0f);
  std::mt19937_64 rng(h->seed ^ 0x6e70726f6265ull);
  auto fill = [&](int off, int fan_in, int count) {
    float b = std::sqrt(6.0f / (float)fan_in);
    std::uniform_real_distribution<float> U(-b, b);
    for (int i = 0; i < count; ++i) P[off + i] = U(rng);
  };
  fill(0, kF, kH1 * kF);
  fill(kH1 * kF + kH1, kH1, kH2 * kH1);
  fill(kH1 * kF + kH1 + kH2 * kH1 + kH2, kH2, kH2);
  double lab_mean = 0, lab_max = 0;
  for (int64_t i = 0; i < N_fit; ++i) {
    lab_mean += hl[i];
    lab_max = std::max<double>(lab_max, hl[i]);
  }
  lab_mean /= N_fit;
  P[np - 1] = (float)lab_mean;  // output bias starts at the mean label
  HORA_TRY(md->params.reserve(4 * np));
  HORA_TRY(md->mean.reserve(4 * kF));
  HORA_TRY(md->inv_std.reserve(4 * kF));
  HORA_CUDA_TRY(cudaMemcpyAsync(md->params.ptr, P.data(), 4 * np, cudaMemcpyHostToDevice, s));
  HORA_CUDA_TRY(cudaMemcpyAsync(md->mean.ptr, mean.data(), 4 * kF, cudaMemcpyHostToDevice, s));
  HORA_CUDA_TRY(cudaMemcpyAsync(md->inv_std.ptr, inv.data(), 4 * kF, cudaMemcpyHostToDevice, s));
  DevBuf mom, var, gp, lp, perm;
  HORA_TRY(mom.reserve(4 * np));
  HORA_TRY(var.reserve(4 * np));
  HORA_TRY(perm.reserve(4 * N_fit));
  HORA_CUDA_TRY(cudaMemsetAsync(mom.ptr, 0, 4 * np, s));
  HORA_CUDA_TRY(cudaMemsetAsync(var.ptr, 0, 4 * np, s));
  const int64_t step_n = 4096;
  const float alpha = 3.0f;  // under-predicting nprobe loses recall
  std::vector<int> order(N_fit);
  std::iota(order.begin(), order.end(), 0);
  int step = 0;
  for (uint64_t ep = 0; ep < epochs; ++ep) {
    std::shuffle(order.begin(), order.end(), rng);
    HORA_CUDA_TRY(cudaMemcpyAsync(perm.ptr, order.data(), 4 * N_fit, cudaMemcpyHostToDevice, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    const float lr = 3e-3f * (ep + 1 < epochs ? 1.0f : 0.3f);
    for (int64_t b = 0; b + step_n <= N_fit || (b == 0 && N_fit < step_n); b += step_n) {
      const int64_t nb = std::min(step_n, N_fit - b);
      ++step;
      HORA_TRY(mlp_step(md->params.as<float>(), kF, kH1, kH2, feats.as<float>(), labels.as<float>(),
                        perm.as<int>() + b, nb, alpha, gp, lp, nullptr, mom.as<float>(), var.as<float>(),
                        step, lr, md->params.as<float>(), s));
    }
  }
  // final loss over the fitted queries
  HORA_TRY(mlp_step(md->params.as<float>(), kF, kH1, kH2, feats.as<float>(), labels.as<float>(), nullptr,
                    N_fit, alpha, gp, lp, nullptr, nullptr, nullptr, 0, 0.0f, nullptr, s));
  const int Gc = ceil_div(N_fit, kMlpBatch);
  std::vector<float> l(Gc);
  HORA_CUDA_TRY(cudaMemcpyAsync(l.data(), lp.ptr, 4 * Gc, cudaMemcpyDeviceToHost, s));
  HORA_CUDA_TRY(cudaStreamSynchronize(s));
  double loss = 0;
  for (float v : l) loss += v;
  loss /= N_fit;
  md->pmax = pm;
  md->p1 = p1;
  md->final_loss = loss;
  md->target = recall_target;
  // margin calibration on the held-out queries: per margin on a 1/32 grid,
  // each query's nprobe as the search computes it, and its recall taken from
  // the hits measured at the largest grid nprobe not above that (nprobe 3 is
  // scored as 2); the smallest margin whose held-out recall@10 reaches the
  // target (less two standard errors) wins
  if (n_cal > 0) {
    DevBuf pred;
    HORA_TRY(pred.reserve(4 * n_cal));
    HORA_TRY(mlp_forward(md->params.as<float>(), kF, kH1, kH2, feats.as<float>() + N_fit * kF, n_cal, nullptr,
                         nullptr, pred.as<float>(), s));
    std::vector<float> hp(n_cal);
    HORA_CUDA_TRY(cudaMemcpyAsync(hp.data(), pred.ptr, 4 * n_cal, cudaMemcpyDeviceToHost, s));
    HORA_CUDA_TRY(cudaStreamSynchronize(s));
    const int hi = std::min(pw, h->nprobe_max > 0 ? h->nprobe_max : pm);
    const int lo = std::max(1, p1);
    bool found = false;
    for (int mi = -160; mi <= 160 && !found; ++mi) {
      const float m = (float)mi / 32.0f;
      double hit = 0, hit2 = 0, probes = 0;
      for (int64_t i = 0; i < n_cal; ++i) {
        float e = std::min(hp[i] + m, 20.0f);
        int p = (int)std::ceil(std::exp2(e) - 1e-4f);
        p = std::min(std::max(p, lo), std::max(hi, lo));
        int gi = 0;
        while (gi + 1 < ng && grid[gi + 1] <= p) ++gi;
        const double r = hh[(size_t)(N_fit + i) * ng + gi] / 10.0;
        hit += r;
        hit2 += r * r;
        probes += p;
      }
      // the held-out recall must clear the target by two standard errors of
      // its mean (per-query recalls), so that other queries of the same law
      // land at or above the target
      const double rec = hit / (double)n_cal;
      const double var = std::max(0.0, hit2 / (double)n_cal - rec * rec);
      const double se = std::sqrt(var / (double)n_cal);
      if (rec - 2.0 * se >= recall_target || mi == 160) {
        md->margin = m;
        md->cal_recall = rec;
        md->cal_nprobe = probes / (double)n_cal;
        found = true;
      }
    }
    md->cal_queries = n_cal;
  }
  h->nprobe = std::move(md);
  if (stats_out) {
    stats_out[0] = loss;
    stats_out[1] = lab_mean;
    stats_out[2] = lab_max;
    stats_out[3] = (double)epochs;
  }
  return HORA_OK;
}

}  // extern "C"
