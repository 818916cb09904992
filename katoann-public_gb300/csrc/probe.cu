// Learned per-query probe budget: features, the MLP that picks each query's
// nprobe, and the kernels that train it.
//
// The reference probes the same number of lists for every query of a batch
// (SearchParams::nprobe, include/katoann/index.h:53; the selection at
// src/index.cpp:864-870). Queries differ in how many lists they need before
// their true neighbours are all probed, and the shape of a query's sorted
// coarse distances (how fast they grow past the nearest list) predicts it.
// A 64 -> 256 -> 256 -> C MLP reads 64 features of that shape and gives a
// distribution over a ladder of nprobe values; the budget is the smallest
// value whose cumulative probability reaches a threshold. Training labels
// are the smallest ladder value whose fixed-nprobe result recovers the
// query's exact top-k (made by the host library from searches).
//
// Inference runs inside the search pipeline: probe_features_kernel (one warp
// per query) and probe_mlp_kernel (one CTA per 32 queries; bf16 weights read
// through L2, activations in shared memory, fp32 accumulation).
// Training uses a tiled fp32 GEMM kernel with generic strides, softmax
// cross-entropy, and Adam on fp32 masters with bf16 copies for the forward
// pass.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "kcommon.cuh"
#include "probe.cuh"

namespace kato {

namespace {

constexpr uint32_t kF = KATO_PROBE_FEATURES;  // 64
constexpr uint32_t kH = KATO_PROBE_HIDDEN;    // 256
constexpr uint32_t kCMax = KATO_PROBE_MAX_CLASSES;
constexpr uint32_t kQB = 16;   // queries per MLP CTA
constexpr uint32_t kAS = 20;   // shared-memory row stride of the activations (floats; 16-byte
                               // rows, conflict-free 128-bit stores)

__device__ __forceinline__ float bf16_value(uint16_t b) {
  return __uint_as_float(static_cast<uint32_t>(b) << 16);
}

// Round-to-nearest-even fp32 -> bf16 (finite values).
__host__ __device__ __forceinline__ uint16_t bf16_round(float f) {
  uint32_t u;
#ifdef __CUDA_ARCH__
  u = __float_as_uint(f);
#else
  std::memcpy(&u, &f, 4);
#endif
  u += 0x7FFFu + ((u >> 16) & 1u);
  return static_cast<uint16_t>(u >> 16);
}

// ------------------------------------------------------------------ features
__global__ void __launch_bounds__(256) probe_features_kernel(
    const float *__restrict__ cd, uint32_t L, const uint32_t *__restrict__ probed, uint32_t P,
    const uint32_t *__restrict__ rank, uint32_t B, float *__restrict__ z) {
  const uint32_t q = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (q >= B) return;
  const float *row = cd + static_cast<size_t>(q) * L;
  const uint32_t *pr = probed + static_cast<size_t>(q) * P;
  // ranks past the selection depth read its last list
  const float d0 = row[pr[0]];
  const float dl = row[pr[min(rank[kF - 1], P - 1)]];
  const float e = 1e-4f * dl + 1e-30f;
  const float l0 = logf(d0 + e);
  for (uint32_t j = lane; j < kF; j += 32) {
    const float d = row[pr[min(rank[j], P - 1)]];
    z[static_cast<size_t>(q) * kF + j] = j == 0 ? l0 : logf(d + e) - l0;
  }
}

// ----------------------------------------------------------------- inference
struct MlpArgs {
  const float *shift, *scale;
  const uint16_t *w1, *w2, *w3;
  const float *b1, *b2, *b3;
  const uint32_t *ladder;
  uint32_t C;
  float threshold;
};

// One dense ReLU layer over the CTA's 16 queries: thread j owns output unit j.
// in: [K][kAS] (unit-major, query fastest), out: [kH][kAS]; w is K x kH bf16
// (global memory through L2, or shared memory).
template <uint32_t K>
__device__ __forceinline__ void dense_relu(const float *in, const uint16_t *__restrict__ w,
                                           const float *__restrict__ b, float *out) {
  const uint32_t j = threadIdx.x;
  float acc[kQB];
  const float bj = b[j];
#pragma unroll
  for (uint32_t i = 0; i < kQB; ++i) acc[i] = bj;
#pragma unroll 8
  for (uint32_t k = 0; k < K; ++k) {
    const float wk = bf16_value(w[k * kH + j]);
    const float4 *x = reinterpret_cast<const float4 *>(in + k * kAS);
#pragma unroll
    for (uint32_t v = 0; v < kQB / 4; ++v) {
      const float4 t = x[v];
      acc[4 * v + 0] = fmaf(wk, t.x, acc[4 * v + 0]);
      acc[4 * v + 1] = fmaf(wk, t.y, acc[4 * v + 1]);
      acc[4 * v + 2] = fmaf(wk, t.z, acc[4 * v + 2]);
      acc[4 * v + 3] = fmaf(wk, t.w, acc[4 * v + 3]);
    }
  }
  float4 *o = reinterpret_cast<float4 *>(out + j * kAS);
#pragma unroll
  for (uint32_t v = 0; v < kQB / 4; ++v)
    o[v] = make_float4(fmaxf(acc[4 * v], 0.f), fmaxf(acc[4 * v + 1], 0.f),
                       fmaxf(acc[4 * v + 2], 0.f), fmaxf(acc[4 * v + 3], 0.f));
}

// activations (x0, h1, h2), logits, then w1 and w3 staged as bf16
constexpr size_t kMlpAct = (static_cast<size_t>(kF) + 2 * kH) * kAS * 4 + kQB * (kCMax + 1) * 4;
constexpr size_t kMlpSmem = kMlpAct + (static_cast<size_t>(kF) * kH + kH * kCMax) * 2;

__global__ void __launch_bounds__(kH) probe_mlp_kernel(const float *__restrict__ z, uint32_t B,
                                                        MlpArgs m, uint32_t cap,
                                                        float *__restrict__ probs,
                                                        uint32_t *__restrict__ nprobe) {
  extern __shared__ __align__(16) float sm[];
  float *x0 = sm;                 // [kF][kAS]
  float *h1 = x0 + kF * kAS;      // [kH][kAS]
  float *h2 = h1 + kH * kAS;      // [kH][kAS]
  float *lg = h2 + kH * kAS;      // [kQB][kCMax + 1]
  uint16_t *sw1 = reinterpret_cast<uint16_t *>(reinterpret_cast<unsigned char *>(sm) + kMlpAct);
  uint16_t *sw3 = sw1 + kF * kH;  // [kH][C]
  const uint32_t q0 = blockIdx.x * kQB, t = threadIdx.x;
  // the first and last layers' weights into shared memory (16-byte copies;
  // w1 is 32 KB, w3 at most 16 KB); the middle layer's 128 KB stream from L2
  {
    const uint4 *g1 = reinterpret_cast<const uint4 *>(m.w1);
    uint4 *s1 = reinterpret_cast<uint4 *>(sw1);
    for (uint32_t i = t; i < kF * kH / 8; i += blockDim.x) s1[i] = g1[i];
    for (uint32_t i = t; i < kH * m.C; i += blockDim.x) sw3[i] = m.w3[i];
  }
  for (uint32_t idx = t; idx < kQB * kF; idx += blockDim.x) {
    const uint32_t i = idx / kF, f = idx % kF;
    float v = 0.f;
    if (q0 + i < B) v = (z[static_cast<size_t>(q0 + i) * kF + f] - m.shift[f]) * m.scale[f];
    x0[f * kAS + i] = v;
  }
  __syncthreads();
  dense_relu<kF>(x0, sw1, m.b1, h1);
  __syncthreads();
  dense_relu<kH>(h1, m.w2, m.b2, h2);
  __syncthreads();
  {
    // logits: thread = (query t / 16, classes t % 16 + 16 u)
    const uint32_t qi = t >> 4, part = t & 15;
    float acc[kCMax / 16];
#pragma unroll
    for (uint32_t u = 0; u < kCMax / 16; ++u) {
      const uint32_t c = part + 16 * u;
      acc[u] = c < m.C ? m.b3[c] : 0.f;
    }
#pragma unroll 4
    for (uint32_t k = 0; k < kH; ++k) {
      const float x = h2[k * kAS + qi];
#pragma unroll
      for (uint32_t u = 0; u < kCMax / 16; ++u) {
        const uint32_t c = part + 16 * u;
        if (c < m.C) acc[u] = fmaf(bf16_value(sw3[k * m.C + c]), x, acc[u]);
      }
    }
#pragma unroll
    for (uint32_t u = 0; u < kCMax / 16; ++u) {
      const uint32_t c = part + 16 * u;
      if (c < m.C) lg[qi * (kCMax + 1) + c] = acc[u];
    }
  }
  __syncthreads();
  if (t < kQB && q0 + t < B) {
    const float *l = lg + t * (kCMax + 1);
    float mx = l[0];
    for (uint32_t c = 1; c < m.C; ++c) mx = fmaxf(mx, l[c]);
    float sum = 0.f;
    for (uint32_t c = 0; c < m.C; ++c) sum += expf(l[c] - mx);
    const float inv = 1.f / sum;
    uint32_t pick = m.C - 1;
    bool found = false;
    float cum = 0.f;
    for (uint32_t c = 0; c < m.C; ++c) {
      const float pc = expf(l[c] - mx) * inv;
      cum += pc;
      if (!found && cum >= m.threshold) {
        pick = c;
        found = true;
      }
      if (probs) probs[static_cast<size_t>(q0 + t) * m.C + c] = pc;
    }
    if (nprobe) nprobe[q0 + t] = max(1u, min(m.ladder[pick], cap));
  }
}

__global__ void clamp_budget_kernel(const uint32_t *__restrict__ in, uint32_t B, uint32_t cap,
                                    uint32_t *__restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < B) out[q] = in ? max(1u, min(in[q], cap)) : cap;
}

// ------------------------------------------------------------------ training
// C[m][n] = sum_k A(m, k) B(k, n) (+ bias[n]) (ReLU), with A(m, k) =
// A[m * sam + k * sak] and B(k, n) = B[k * sbk + n * sbn]; C row-major (ldc).
// 64 x 64 tiles, 16-deep slices, 4 x 4 outputs per thread.
template <typename TB>
__device__ __forceinline__ float load_b(const TB *p) {
  if constexpr (sizeof(TB) == 2) return bf16_value(*p);
  else return *p;
}

template <typename TB>
__global__ void __launch_bounds__(256) gemm_kernel(uint32_t M, uint32_t N, uint32_t K,
                                                   const float *__restrict__ A, size_t sam,
                                                   size_t sak, const TB *__restrict__ Bm,
                                                   size_t sbk, size_t sbn, float *__restrict__ C,
                                                   size_t ldc, const float *__restrict__ bias,
                                                   int relu) {
  __shared__ float As[16][64 + 4], Bs[16][64 + 4];
  const uint32_t tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const uint32_t m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (uint32_t k0 = 0; k0 < K; k0 += 16) {
    for (uint32_t i = threadIdx.x; i < 16 * 64; i += 256) {
      // the unit-stride index fastest across threads, for coalesced loads
      uint32_t kk, mm;
      if (sak == 1) { kk = i & 15; mm = i >> 4; } else { mm = i & 63; kk = i >> 6; }
      const uint32_t gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[gm * sam + gk * sak] : 0.f;
      uint32_t kb, nn;
      if (sbk == 1) { kb = i & 15; nn = i >> 4; } else { nn = i & 63; kb = i >> 6; }
      const uint32_t gn = n0 + nn, gkb = k0 + kb;
      Bs[kb][nn] = (gn < N && gkb < K) ? load_b(Bm + gkb * sbk + gn * sbn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        a[r] = As[kk][ty * 4 + r];
        b[r] = Bs[kk][tx * 4 + r];
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const uint32_t gm = m0 + ty * 4 + r, gn = n0 + tx * 4 + c;
      if (gm < M && gn < N) {
        float v = acc[r][c] + (bias ? bias[gn] : 0.f);
        if (relu) v = fmaxf(v, 0.f);
        C[gm * ldc + gn] = v;
      }
    }
}

__global__ void relu_backward_kernel(float *__restrict__ g, const float *__restrict__ h, size_t n) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n && !(h[i] > 0.f)) g[i] = 0.f;
}

// out[c] = sum over rows of g[r][c] (one thread per column, rows in order).
__global__ void colsum_kernel(const float *__restrict__ g, uint32_t rows, uint32_t cols,
                              float *__restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (uint32_t r = 0; r < rows; ++r) s += g[static_cast<size_t>(r) * cols + c];
  out[c] = s;
}

// Softmax cross-entropy per row: dlogits = (softmax - onehot) / n; the loss
// of each row into row_loss.
__global__ void xent_kernel(const float *__restrict__ lg, const uint8_t *__restrict__ label,
                            uint32_t n, uint32_t C, float inv_n, float *__restrict__ dlg,
                            float *__restrict__ row_loss) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float *l = lg + static_cast<size_t>(r) * C;
  float mx = l[0];
  for (uint32_t c = 1; c < C; ++c) mx = fmaxf(mx, l[c]);
  float sum = 0.f;
  for (uint32_t c = 0; c < C; ++c) sum += expf(l[c] - mx);
  const uint32_t y = min(static_cast<uint32_t>(label[r]), C - 1);  // labels past C: the last class
  for (uint32_t c = 0; c < C; ++c) {
    const float p = expf(l[c] - mx) / sum;
    dlg[static_cast<size_t>(r) * C + c] = (p - (c == y ? 1.f : 0.f)) * inv_n;
  }
  row_loss[r] = logf(sum) + mx - l[y];
}

// Sum of a vector by one CTA (fixed order: deterministic).
__global__ void __launch_bounds__(256) sum_kernel(const float *__restrict__ x, uint32_t n,
                                                  float *__restrict__ out) {
  __shared__ double part[256];
  double s = 0;
  for (uint32_t i = threadIdx.x; i < n; i += 256) s += x[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t w = 128; w; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = static_cast<float>(part[0]);
}

// Adam with decoupled weight decay; refreshes the bf16 copy when given.
__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g,
                            float *__restrict__ m1, float *__restrict__ m2, uint32_t n, float lr,
                            float c1, float c2, float wd, uint16_t *__restrict__ wh) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = 0.9f * m1[i] + 0.1f * gi;
  const float b = 0.999f * m2[i] + 0.001f * gi * gi;
  m1[i] = a;
  m2[i] = b;
  float v = w[i] * (1.f - lr * wd);
  v -= lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
  w[i] = v;
  if (wh) wh[i] = bf16_round(v);
}

__global__ void to_bf16_kernel(const float *__restrict__ w, uint32_t n, uint16_t *__restrict__ wh) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wh[i] = bf16_round(w[i]);
}

// Mean and 1 / standard deviation of every feature column (one CTA each).
__global__ void __launch_bounds__(256) feature_stats_kernel(const float *__restrict__ z, uint32_t n,
                                                            float *__restrict__ shift,
                                                            float *__restrict__ scale) {
  __shared__ double part[256];
  const uint32_t f = blockIdx.x;
  double s = 0;
  for (uint32_t i = threadIdx.x; i < n; i += 256) s += z[static_cast<size_t>(i) * kF + f];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t w = 128; w; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  const double mean = part[0] / n;
  __syncthreads();
  double v = 0;
  for (uint32_t i = threadIdx.x; i < n; i += 256) {
    const double d = z[static_cast<size_t>(i) * kF + f] - mean;
    v += d * d;
  }
  part[threadIdx.x] = v;
  __syncthreads();
  for (uint32_t w = 128; w; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double sd = sqrt(part[0] / n);
    shift[f] = static_cast<float>(mean);
    scale[f] = static_cast<float>(1.0 / (sd > 1e-6 ? sd : 1e-6));
  }
}

// Rows perm[0..nb) of z, standardized, and their labels.
__global__ void gather_batch_kernel(const float *__restrict__ z, const uint8_t *__restrict__ label,
                                    const uint32_t *__restrict__ perm, uint32_t nb,
                                    const float *__restrict__ shift, const float *__restrict__ scale,
                                    float *__restrict__ x, uint8_t *__restrict__ y) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb * kF) return;
  const uint32_t r = i / kF, f = i % kF, src = perm[r];
  x[i] = (z[static_cast<size_t>(src) * kF + f] - shift[f]) * scale[f];
  if (f == 0) y[r] = label[src];
}

// --------------------------------------------------- forward and backward
struct Weights {  // what the forward pass reads
  const uint16_t *w1, *w2, *w3;
  const float *b1, *b2, *b3;
};

struct Grads {
  float *w1, *b1, *w2, *b2, *w3, *b3;
};

struct Acts {  // per-batch activations and their gradients (nb rows)
  float *h1, *h2, *lg, *dlg, *d2, *d1, *rowloss, *loss;
};

template <typename TB>
int gemm(uint32_t M, uint32_t N, uint32_t K, const float *A, size_t sam, size_t sak, const TB *B,
         size_t sbk, size_t sbn, float *C, size_t ldc, const float *bias, bool relu,
         cudaStream_t st) {
  const dim3 grid(div_up(N, 64), div_up(M, 64));
  gemm_kernel<TB><<<grid, 256, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, relu);
  KATO_LAUNCHED("gemm_kernel");
  return KATO_OK;
}

// Loss and gradients of one batch x (nb x 64, standardized) with labels y.
int forward_backward(const Weights &w, const float *x, const uint8_t *y, uint32_t nb, uint32_t C,
                     const Acts &a, const Grads &g, cudaStream_t st) {
  int rc;
  // forward
  if ((rc = gemm<uint16_t>(nb, kH, kF, x, kF, 1, w.w1, kH, 1, a.h1, kH, w.b1, true, st))) return rc;
  if ((rc = gemm<uint16_t>(nb, kH, kH, a.h1, kH, 1, w.w2, kH, 1, a.h2, kH, w.b2, true, st))) return rc;
  if ((rc = gemm<uint16_t>(nb, C, kH, a.h2, kH, 1, w.w3, C, 1, a.lg, C, w.b3, false, st))) return rc;
  xent_kernel<<<div_up(nb, 256), 256, 0, st>>>(a.lg, y, nb, C, 1.f / nb, a.dlg, a.rowloss);
  sum_kernel<<<1, 256, 0, st>>>(a.rowloss, nb, a.loss);
  KATO_LAUNCHED("loss kernels");
  // layer 3: gW3 = H2^T dLG, gb3 = colsum dLG, d2 = dLG W3^T (masked by H2 > 0)
  if ((rc = gemm<float>(kH, C, nb, a.h2, 1, kH, a.dlg, C, 1, g.w3, C, nullptr, false, st))) return rc;
  colsum_kernel<<<div_up(C, 128), 128, 0, st>>>(a.dlg, nb, C, g.b3);
  if ((rc = gemm<uint16_t>(nb, kH, C, a.dlg, C, 1, w.w3, 1, C, a.d2, kH, nullptr, false, st))) return rc;
  const size_t nh = static_cast<size_t>(nb) * kH;
  relu_backward_kernel<<<static_cast<uint32_t>((nh + 255) / 256), 256, 0, st>>>(a.d2, a.h2, nh);
  // layer 2
  if ((rc = gemm<float>(kH, kH, nb, a.h1, 1, kH, a.d2, kH, 1, g.w2, kH, nullptr, false, st))) return rc;
  colsum_kernel<<<div_up(kH, 128), 128, 0, st>>>(a.d2, nb, kH, g.b2);
  if ((rc = gemm<uint16_t>(nb, kH, kH, a.d2, kH, 1, w.w2, 1, kH, a.d1, kH, nullptr, false, st))) return rc;
  relu_backward_kernel<<<static_cast<uint32_t>((nh + 255) / 256), 256, 0, st>>>(a.d1, a.h1, nh);
  // layer 1
  if ((rc = gemm<float>(kF, kH, nb, x, 1, kF, a.d1, kH, 1, g.w1, kH, nullptr, false, st))) return rc;
  colsum_kernel<<<div_up(kH, 128), 128, 0, st>>>(a.d1, nb, kH, g.b1);
  KATO_LAUNCHED("backward kernels");
  return KATO_OK;
}

// A device allocation freed on scope exit.
struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double uniform01(uint64_t &s) { return static_cast<double>(splitmix(s) >> 11) * 0x1.0p-53; }

}  // namespace

int check_probe_model(const katoann_gpu_probe_model &m) {
  if (m.nclass < 2 || m.nclass > kCMax) return invalid("probe model: 2 to 32 classes");
  if (m.depth == 0 || m.depth > 4096) return invalid("probe model: depth must be 1 to 4096");
  if (!m.d_rank || !m.d_shift || !m.d_scale || !m.d_w1 || !m.d_b1 || !m.d_w2 || !m.d_b2 ||
      !m.d_w3 || !m.d_b3 || !m.d_ladder)
    return invalid("probe model: null array");
  if (reinterpret_cast<uintptr_t>(m.d_w1) % 16)
    return invalid("probe model: d_w1 must be 16-byte aligned");
  return KATO_OK;
}

int probe_features(const float *cd, uint32_t L, const uint32_t *probed, uint32_t P,
                   const uint32_t *rank, uint32_t B, float *z, cudaStream_t st) {
  if (B == 0) return KATO_OK;
  probe_features_kernel<<<div_up(B, 8), 256, 0, st>>>(cd, L, probed, P, rank, B, z);
  KATO_LAUNCHED("probe_features_kernel");
  return KATO_OK;
}

int probe_budget(const katoann_gpu_probe_model &m, const float *z, uint32_t B, uint32_t cap,
                 float *probs, uint32_t *nprobe, cudaStream_t st) {
  if (B == 0) return KATO_OK;
  if (const int rc = smem_limit(reinterpret_cast<const void *>(probe_mlp_kernel),
                                static_cast<int>(kMlpSmem), "probe_mlp_kernel shared memory"))
    return rc;
  const MlpArgs a{m.d_shift, m.d_scale, m.d_w1, m.d_w2, m.d_w3, m.d_b1,
                  m.d_b2,    m.d_b3,    m.d_ladder, m.nclass, m.threshold};
  probe_mlp_kernel<<<div_up(B, kQB), kH, kMlpSmem, st>>>(z, B, a, cap, probs, nprobe);
  KATO_LAUNCHED("probe_mlp_kernel");
  return KATO_OK;
}

int clamp_budget(const uint32_t *in, uint32_t B, uint32_t cap, uint32_t *out, cudaStream_t st) {
  if (B == 0) return KATO_OK;
  clamp_budget_kernel<<<div_up(B, 256), 256, 0, st>>>(in, B, cap, out);
  KATO_LAUNCHED("clamp_budget_kernel");
  return KATO_OK;
}

// Bytes of every training buffer for batches of nb rows and C classes.
namespace {

struct TrainLayout {
  size_t x, y, perm, h1, h2, lg, dlg, d2, d1, rowloss, loss, g, total;
};

TrainLayout train_layout(uint32_t nb, uint32_t C, uint32_t n) {
  TrainLayout t{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += (bytes + 255) / 256 * 256;
    return at;
  };
  t.x = take(static_cast<size_t>(nb) * kF * 4);
  t.y = take(nb);
  t.perm = take(static_cast<size_t>(n) * 4);
  t.h1 = take(static_cast<size_t>(nb) * kH * 4);
  t.h2 = take(static_cast<size_t>(nb) * kH * 4);
  t.lg = take(static_cast<size_t>(nb) * C * 4);
  t.dlg = take(static_cast<size_t>(nb) * C * 4);
  t.d2 = take(static_cast<size_t>(nb) * kH * 4);
  t.d1 = take(static_cast<size_t>(nb) * kH * 4);
  t.rowloss = take(static_cast<size_t>(nb) * 4);
  t.loss = take(static_cast<size_t>(n / std::max(nb, 1u) + 2) * 4);
  t.g = take((static_cast<size_t>(kF) * kH + kH + kH * kH + kH + kH * C + C) * 4);
  t.total = o;
  return t;
}

Grads grads_at(float *g, uint32_t C) {
  Grads r{};
  r.w1 = g;
  r.b1 = r.w1 + kF * kH;
  r.w2 = r.b1 + kH;
  r.b2 = r.w2 + kH * kH;
  r.w3 = r.b2 + kH;
  r.b3 = r.w3 + kH * C;
  return r;
}

}  // namespace

static int probe_train(const float *z, const uint8_t *label, uint32_t n, uint32_t C,
                const katoann_gpu_probe_train_options &opt, float *shift, float *scale, float *w1,
                float *b1, float *w2, float *b2, float *w3, float *b3, float *loss) {
  if (n == 0 || C < 2 || C > kCMax) return invalid("probe training: need rows and 2 to 32 classes");
  if (opt.epochs == 0 || opt.batch == 0 || opt.batch > 65536 || !(opt.lr > 0.f))
    return invalid("probe training: bad options");
  const uint32_t nb = std::min(opt.batch, n);
  const size_t P = static_cast<size_t>(kF) * kH + kH + kH * kH + kH + kH * C + C;  // parameters
  const TrainLayout tl = train_layout(nb, C, n);
  DevBuf work, params;
  // params: fp32 masters, Adam moments (2x), bf16 copies of the weights, the standardization
  const size_t pbytes = P * 4 * 3 + P * 2 + 2 * kF * 4 + 1024;
  KATO_CUDA(cudaMalloc(&work.p, tl.total));
  KATO_CUDA(cudaMalloc(&params.p, pbytes));
  unsigned char *wb = static_cast<unsigned char *>(work.p);
  float *master = static_cast<float *>(params.p);
  float *mom1 = master + P, *mom2 = mom1 + P;
  uint16_t *half = reinterpret_cast<uint16_t *>(mom2 + P);
  float *d_shift = reinterpret_cast<float *>(half + P + (P & 1));
  float *d_scale = d_shift + kF;
  cudaStream_t st = nullptr;
  // initial weights: uniform(+-sqrt(6 / inputs)), biases zero
  std::vector<float> init(P, 0.f);
  uint64_t s = opt.seed * 0x9E3779B97F4A7C15ull + 12345;
  const Grads mp = grads_at(init.data(), C);
  auto fill = [&](float *p, size_t cnt, uint32_t fan_in) {
    const double a = std::sqrt(6.0 / fan_in);
    for (size_t i = 0; i < cnt; ++i) p[i] = static_cast<float>((2 * uniform01(s) - 1) * a);
  };
  fill(mp.w1, kF * kH, kF);
  fill(mp.w2, kH * kH, kH);
  fill(mp.w3, kH * C, kH);
  KATO_CUDA(cudaMemcpy(master, init.data(), P * 4, cudaMemcpyHostToDevice));
  KATO_CUDA(cudaMemset(mom1, 0, P * 8));
  to_bf16_kernel<<<static_cast<uint32_t>((P + 255) / 256), 256, 0, st>>>(master, P, half);
  feature_stats_kernel<<<kF, 256, 0, st>>>(z, n, d_shift, d_scale);
  KATO_LAUNCHED("probe training setup");
  const Grads m = grads_at(master, C);
  const Weights w{half + (m.w1 - master), half + (m.w2 - master), half + (m.w3 - master),
                  m.b1, m.b2, m.b3};
  float *x = reinterpret_cast<float *>(wb + tl.x);
  uint8_t *y = wb + tl.y;
  uint32_t *perm = reinterpret_cast<uint32_t *>(wb + tl.perm);
  const Acts a{reinterpret_cast<float *>(wb + tl.h1),  reinterpret_cast<float *>(wb + tl.h2),
               reinterpret_cast<float *>(wb + tl.lg),  reinterpret_cast<float *>(wb + tl.dlg),
               reinterpret_cast<float *>(wb + tl.d2),  reinterpret_cast<float *>(wb + tl.d1),
               reinterpret_cast<float *>(wb + tl.rowloss), reinterpret_cast<float *>(wb + tl.loss)};
  const Grads g = grads_at(reinterpret_cast<float *>(wb + tl.g), C);
  const uint32_t steps = n / nb;  // full batches per epoch (the rest joins the next shuffle)
  std::vector<uint32_t> order(n);
  std::vector<float> step_loss(steps + 1);
  uint64_t t = 0;
  int rc;
  for (uint32_t e = 0; e < opt.epochs; ++e) {
    for (uint32_t i = 0; i < n; ++i) order[i] = i;
    for (uint32_t i = n - 1; i > 0; --i) std::swap(order[i], order[splitmix(s) % (i + 1)]);
    KATO_CUDA(cudaMemcpyAsync(perm, order.data(), static_cast<size_t>(n) * 4,
                              cudaMemcpyHostToDevice, st));
    for (uint32_t b = 0; b < steps; ++b) {
      gather_batch_kernel<<<div_up(nb * kF, 256), 256, 0, st>>>(z, label, perm + b * nb, nb,
                                                                d_shift, d_scale, x, y);
      Acts ab = a;
      ab.loss = a.loss + b;
      if ((rc = forward_backward(w, x, y, nb, C, ab, g, st))) return rc;
      ++t;
      const float c1 = 1.f - std::pow(0.9f, static_cast<float>(t));
      const float c2 = 1.f - std::pow(0.999f, static_cast<float>(t));
      // weights (with decay and bf16 refresh), then biases (no decay)
      auto step = [&](float *wp, const float *gp, size_t cnt, bool weight) {
        const size_t at = wp - master;
        adam_kernel<<<static_cast<uint32_t>((cnt + 255) / 256), 256, 0, st>>>(
            wp, gp, mom1 + at, mom2 + at, static_cast<uint32_t>(cnt), opt.lr, c1, c2,
            weight ? opt.weight_decay : 0.f, weight ? half + at : nullptr);
      };
      step(m.w1, g.w1, kF * kH, true);
      step(m.b1, g.b1, kH, false);
      step(m.w2, g.w2, kH * kH, true);
      step(m.b2, g.b2, kH, false);
      step(m.w3, g.w3, kH * C, true);
      step(m.b3, g.b3, C, false);
      KATO_LAUNCHED("adam_kernel");
    }
    KATO_CUDA(cudaMemcpyAsync(step_loss.data(), a.loss, steps * 4, cudaMemcpyDeviceToHost, st));
    KATO_CUDA(cudaStreamSynchronize(st));
    double sum = 0;
    for (uint32_t b = 0; b < steps; ++b) sum += step_loss[b] / nb;
    if (loss) loss[e] = static_cast<float>(sum / std::max(steps, 1u));
  }
  KATO_CUDA(cudaMemcpy(shift, d_shift, kF * 4, cudaMemcpyDeviceToHost));
  KATO_CUDA(cudaMemcpy(scale, d_scale, kF * 4, cudaMemcpyDeviceToHost));
  KATO_CUDA(cudaMemcpy(w1, m.w1, kF * kH * 4, cudaMemcpyDeviceToHost));
  KATO_CUDA(cudaMemcpy(b1, m.b1, kH * 4, cudaMemcpyDeviceToHost));
  KATO_CUDA(cudaMemcpy(w2, m.w2, kH * kH * 4, cudaMemcpyDeviceToHost));
  KATO_CUDA(cudaMemcpy(b2, m.b2, kH * 4, cudaMemcpyDeviceToHost));
  KATO_CUDA(cudaMemcpy(w3, m.w3, static_cast<size_t>(kH) * C * 4, cudaMemcpyDeviceToHost));
  KATO_CUDA(cudaMemcpy(b3, m.b3, static_cast<size_t>(C) * 4, cudaMemcpyDeviceToHost));
  return KATO_OK;
}

static int probe_grads(const katoann_gpu_probe_model &mdl, const float *z, const uint8_t *label,
                uint32_t n, float *loss, const Grads &out) {
  if (n == 0) return invalid("probe gradients: no rows");
  const uint32_t C = mdl.nclass;
  const TrainLayout tl = train_layout(n, C, n);
  DevBuf work;
  KATO_CUDA(cudaMalloc(&work.p, tl.total));
  unsigned char *wb = static_cast<unsigned char *>(work.p);
  cudaStream_t st = nullptr;
  std::vector<uint32_t> order(n);
  for (uint32_t i = 0; i < n; ++i) order[i] = i;
  uint32_t *perm = reinterpret_cast<uint32_t *>(wb + tl.perm);
  KATO_CUDA(cudaMemcpy(perm, order.data(), static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice));
  float *x = reinterpret_cast<float *>(wb + tl.x);
  uint8_t *y = wb + tl.y;
  gather_batch_kernel<<<div_up(n * kF, 256), 256, 0, st>>>(z, label, perm, n, mdl.d_shift,
                                                           mdl.d_scale, x, y);
  KATO_LAUNCHED("gather_batch_kernel");
  const Acts a{reinterpret_cast<float *>(wb + tl.h1),  reinterpret_cast<float *>(wb + tl.h2),
               reinterpret_cast<float *>(wb + tl.lg),  reinterpret_cast<float *>(wb + tl.dlg),
               reinterpret_cast<float *>(wb + tl.d2),  reinterpret_cast<float *>(wb + tl.d1),
               reinterpret_cast<float *>(wb + tl.rowloss), reinterpret_cast<float *>(wb + tl.loss)};
  const Weights w{mdl.d_w1, mdl.d_w2, mdl.d_w3, mdl.d_b1, mdl.d_b2, mdl.d_b3};
  int rc = forward_backward(w, x, y, n, C, a, out, st);
  if (rc) return rc;
  float sum = 0;
  KATO_CUDA(cudaMemcpy(&sum, a.loss, 4, cudaMemcpyDeviceToHost));
  *loss = sum / n;
  return KATO_OK;
}

}  // namespace kato

using kato::as_stream;

extern "C" {

int katoann_gpu_probe_predict(const katoann_gpu_probe_model *model, const float *d_z, uint32_t n,
                              uint32_t cap, float *d_probs, uint32_t *d_nprobe,
                              katoann_stream_t stream) {
  if (!model) return kato::invalid("null probe model");
  if (int rc = kato::check_probe_model(*model)) return rc;
  if (cap == 0) return kato::invalid("budget cap must be positive");
  return kato::probe_budget(*model, d_z, n, cap, d_probs, d_nprobe, as_stream(stream));
}

int katoann_gpu_probe_train(const float *d_z, const uint8_t *d_label, uint32_t n,
                            uint32_t nclass, const katoann_gpu_probe_train_options *options,
                            float *h_shift, float *h_scale, float *h_w1, float *h_b1, float *h_w2,
                            float *h_b2, float *h_w3, float *h_b3, float *h_loss) {
  if (!options) return kato::invalid("null training options");
  return kato::probe_train(d_z, d_label, n, nclass, *options, h_shift, h_scale, h_w1, h_b1, h_w2,
                           h_b2, h_w3, h_b3, h_loss);
}

int katoann_gpu_probe_grads(const katoann_gpu_probe_model *model, const float *d_z,
                            const uint8_t *d_label, uint32_t n, float *h_loss, float *d_gw1,
                            float *d_gb1, float *d_gw2, float *d_gb2, float *d_gw3,
                            float *d_gb3) {
  if (!model) return kato::invalid("null probe model");
  if (int rc = kato::check_probe_model(*model)) return rc;
  const kato::Grads g{d_gw1, d_gb1, d_gw2, d_gb2, d_gw3, d_gb3};
  return kato::probe_grads(*model, d_z, d_label, n, h_loss, g);
}

}  // extern "C"
