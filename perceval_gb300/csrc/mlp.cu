// Kernels of the learned autoregressive proposal (a small MLP over output modes):
// a BF16 tensor-core GEMM with FP32 accumulation and fused epilogues, and the
// elementwise pieces of its forward, backward and Adam update.
//
// GEMM:  C[m, n] = sum_k A(m, k) B(n, k)   (+ bias[n], then optionally GELU)
//   A(m, k) = transA ? A[k * lda + m] : A[m * lda + k]
//   B(n, k) = transB ? B[k * ldb + n] : B[n * ldb + k]
// so Y = X W^T (forward), dX = dY W (transB), dW = dY^T X (transA, transB) are all one
// kernel with the weight matrices in torch Linear layout (out x in, row-major).
//
// Tiling: 128 x 128 x 32 per CTA, 8 warps of 64 x 32, mma.sync m16n8k16 (bf16 in,
// f32 accumulate) with fragments read from padded shared-memory tiles in the operand
// layouts of the PTX ISA (A row-major 16x16: rows g / g + 8, columns 2t / 2t + 8;
// B column-major 16x8: rows 2t / 2t + 8, column g; C: rows g / g + 8, columns 2t,
// with g = lane / 4 and t = lane % 4).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "runtime.cuh"

namespace pcvl {

constexpr int GBM = 128, GBN = 128, GBK = 32, GPAD = 8;

enum Epilogue { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2 };

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  int M, N, K, lda, ldb, ldc;
  int transA, transB;
  float alpha, beta;          // C = alpha * AB + beta * C (+ epilogue); beta uses ldc
  const float* bias;          // per n (EPI_BIAS*)
  int epi;
  float* C;                   // f32 output (may be null)
  __nv_bfloat16* Cb;          // bf16 copy of the output (may be null), ldc
  float* Cpre;                // pre-activation (f32) for EPI_BIAS_GELU (may be null), ldc
};

// one 128 x 32 operand tile into shared memory as [row][k] (k contiguous)
__device__ __forceinline__ void load_tile(const __nv_bfloat16* __restrict__ G, int trans, int ld, int rows, int K,
                                          int row0, int k0, __nv_bfloat16 (*S)[GBK + GPAD]) {
  const int tid = threadIdx.x;
  if (!trans) {
    // 128 rows x 32 k: 512 chunks of 8 contiguous k; 2 per thread
    for (int c = tid; c < GBM * GBK / 8; c += blockDim.x) {
      const int r = c >> 2, kk = (c & 3) * 8;
      const int gr = row0 + r, gk = k0 + kk;
      __nv_bfloat16 v[8];
      if (gr < rows && gk + 7 < K && ((ld & 7) == 0)) {
        const uint4 q = *reinterpret_cast<const uint4*>(&G[(size_t)gr * ld + gk]);
        *reinterpret_cast<uint4*>(v) = q;
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e)
          v[e] = (gr < rows && gk + e < K) ? G[(size_t)gr * ld + gk + e] : __float2bfloat16(0.f);
      }
#pragma unroll
      for (int e = 0; e < 8; ++e) S[r][kk + e] = v[e];
    }
  } else {
    // element (row, k) at G[k * ld + row]: 32 k x 128 rows, rows contiguous
    for (int c = tid; c < GBM * GBK / 8; c += blockDim.x) {
      const int kk = c >> 4, r = (c & 15) * 8;
      const int gr = row0 + r, gk = k0 + kk;
      __nv_bfloat16 v[8];
      if (gk < K && gr + 7 < rows && ((ld & 7) == 0)) {
        const uint4 q = *reinterpret_cast<const uint4*>(&G[(size_t)gk * ld + gr]);
        *reinterpret_cast<uint4*>(v) = q;
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e)
          v[e] = (gk < K && gr + e < rows) ? G[(size_t)gk * ld + gr + e] : __float2bfloat16(0.f);
      }
#pragma unroll
      for (int e = 0; e < 8; ++e) S[r + e][kk] = v[e];
    }
  }
}

__global__ void __launch_bounds__(256) gemm_bf16_kernel(GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 As[GBM][GBK + GPAD];
  __shared__ __align__(16) __nv_bfloat16 Bs[GBN][GBK + GPAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps of 64 x 32
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const int gq = lane >> 2, tq = lane & 3;
  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

  for (int k0 = 0; k0 < g.K; k0 += GBK) {
    load_tile(g.A, g.transA, g.lda, g.M, g.K, m0, k0, As);
    load_tile(g.B, g.transB, g.ldb, g.N, g.K, n0, k0, Bs);
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < GBK; ks += 16) {
      uint32_t af[4][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = wm * 64 + i * 16 + gq;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * tq]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * tq]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * tq + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn * 32 + j * 8 + gq;
        bf[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * tq]);
        bf[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int r = m0 + wm * 64 + i * 16 + gq + (e >= 2 ? 8 : 0);
        const int c = n0 + wn * 32 + j * 8 + 2 * tq + (e & 1);
        if (r < g.M && c < g.N) {
          const size_t o = (size_t)r * g.ldc + c;
          float v = g.alpha * acc[i][j][e];
          if (g.beta != 0.f) v += g.beta * g.C[o];
          if (g.epi != EPI_NONE) v += g.bias[c];
          if (g.epi == EPI_BIAS_GELU) {
            if (g.Cpre) g.Cpre[o] = v;
            v = gelu_f(v);
          }
          if (g.C) g.C[o] = v;
          if (g.Cb) g.Cb[o] = __float2bfloat16(v);
        }
      }
    }
  }
}

// ---------------------------------------------------------------- elementwise kernels
__global__ void k_gelu_backward(const float* __restrict__ dy, const float* __restrict__ pre, int64_t n,
                                __nv_bfloat16* __restrict__ dxb, float* __restrict__ dx) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = dy[i] * gelu_grad(pre[i]);
    if (dx) dx[i] = v;
    if (dxb) dxb[i] = __float2bfloat16(v);
  }
}

__global__ void k_f32_to_bf16(const float* __restrict__ x, int64_t n, __nv_bfloat16* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

// column sums: out[n] = sum_m x[m * ld + n]   (bias gradients); one thread per column
__global__ void k_colsum(const float* __restrict__ x, int M, int N, int ld, float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f, c = 0.f;
  for (int m = 0; m < M; ++m) {
    const float y = x[(size_t)m * ld + n] - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  out[n] = s;
}

// Row-wise masked log-softmax over N logits.  Row r: logits[r*N .. ], target[r]
// (< 0: row ignored).  Writes logprob of the target (or of every entry when
// `all_logp` is set) and, when grad != null, d(mean NLL)/dlogits = (softmax - onehot)
// * scale.  One warp per row.
__global__ void k_softmax_xent(const float* __restrict__ logits, int R, int N, const int32_t* __restrict__ target,
                               float scale, float* __restrict__ logp_target, float* __restrict__ grad,
                               __nv_bfloat16* __restrict__ gradb, float* __restrict__ all_logp) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= R) return;
  const float* x = logits + (size_t)warp * N;
  float mx = -INFINITY;
  for (int j = lane; j < N; j += 32) mx = fmaxf(mx, x[j]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
  float se = 0.f;
  for (int j = lane; j < N; j += 32) se += expf(x[j] - mx);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) se += __shfl_xor_sync(0xffffffffu, se, d);
  const float lse = mx + logf(se);
  const int t = target ? target[warp] : -1;
  if (lane == 0 && logp_target) logp_target[warp] = t >= 0 ? x[t] - lse : 0.f;
  if (all_logp)
    for (int j = lane; j < N; j += 32) all_logp[(size_t)warp * N + j] = x[j] - lse;
  if (grad || gradb) {
    for (int j = lane; j < N; j += 32) {
      const float pj = expf(x[j] - lse);
      const float gv = t >= 0 ? (pj - (j == t ? 1.f : 0.f)) * scale : 0.f;
      if (grad) grad[(size_t)warp * N + j] = gv;
      if (gradb) gradb[(size_t)warp * N + j] = __float2bfloat16(gv);
    }
  }
}

// Input rows of the proposal network for every (sequence, step), or for one step:
//   h[row] = pos_emb[k] + sum_{l<k} mode_emb[seq[s*n + l]]   (bf16 out, D columns)
// with row = s * n + k (step < 0) or row = s, k = step.
__global__ void k_bag_embed(const int32_t* __restrict__ seq, int S, int n, int step, const float* __restrict__ mode_emb,
                            const float* __restrict__ pos_emb, int D, __nv_bfloat16* __restrict__ h) {
  const int row = blockIdx.x;
  if (row >= (step < 0 ? S * n : S)) return;
  const int s = step < 0 ? row / n : row, k = step < 0 ? row - s * n : step;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    float v = pos_emb[(size_t)k * D + d];
    for (int l = 0; l < k; ++l) v += mode_emb[(size_t)seq[s * n + l] * D + d];
    h[(size_t)row * D + d] = __float2bfloat16(v);
  }
}

// gradients of the embedding tables from dh (f32, rows s*n + k)
__global__ void k_bag_embed_backward(const int32_t* __restrict__ seq, int S, int n, const float* __restrict__ dh,
                                     int D, float* __restrict__ dmode, float* __restrict__ dpos) {
  const int row = blockIdx.x;
  if (row >= S * n) return;
  const int s = row / n, k = row - s * n;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    const float g = dh[(size_t)row * D + d];
    atomicAdd(&dpos[(size_t)k * D + d], g);
    for (int l = 0; l < k; ++l) atomicAdd(&dmode[(size_t)seq[s * n + l] * D + d], g);
  }
}

// Adam (Kingma & Ba 2015) on f32 master weights, refreshing the bf16 copy
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ gr, float* __restrict__ m1,
                       float* __restrict__ m2, int64_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ wb) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g = gr[i];
    const float a = b1 * m1[i] + (1.f - b1) * g;
    const float b = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a;
    m2[i] = b;
    const float v = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[i] = v;
    if (wb) wb[i] = __float2bfloat16(v);
  }
}

// One autoregressive step of proposal sampling for S chains: from f32 logits (S x N),
// draw mode j with probability softmax(logits)_j restricted to modes with capacity
// (cap[j] > 0 for every mode here), with a Philox uniform (key, counter (chain, step));
// accumulates the log-probability of the draw into logq[s] (f64).
__global__ void k_sample_step(const float* __restrict__ logits, int S, int N, int step, uint32_t k0, uint32_t k1,
                              uint64_t chain0, int32_t* __restrict__ seq, int n, double* __restrict__ logq) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= S) return;
  const float* x = logits + (size_t)warp * N;
  float mx = -INFINITY;
  for (int j = lane; j < N; j += 32) mx = fmaxf(mx, x[j]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
  float se = 0.f;
  for (int j = lane; j < N; j += 32) se += expf(x[j] - mx);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) se += __shfl_xor_sync(0xffffffffu, se, d);
  const uint64_t chain = chain0 + (uint64_t)warp;
  const u4 r = philox4x32_10({(uint32_t)chain, (uint32_t)(chain >> 32), (uint32_t)step, 0x51u}, k0, k1);
  const float target = (float)u01_from(r.x, r.y) * se;
  // prefix scan over lanes in chunks of 32 modes
  float run = 0.f;
  int pick = N - 1;
  for (int base = 0; base < N; base += 32) {
    const int j = base + lane;
    float v = j < N ? expf(x[j] - mx) : 0.f;
    float incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, j < N && run + incl > target);
    if (hit) {
      pick = base + __ffs(hit) - 1;
      break;
    }
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) {
    seq[(size_t)warp * n + step] = pick;
    logq[warp] += (double)(x[pick] - mx) - log((double)se);
  }
}

static int grid1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 65536)); }

}  // namespace pcvl

using namespace pcvl;

extern "C" int pcvl_gemm_bf16(const void* A, const void* B, int32_t M, int32_t N, int32_t K, int32_t lda,
                              int32_t ldb, int32_t transA, int32_t transB, float alpha, float beta,
                              const float* bias, int32_t epilogue, float* C, void* Cb, float* Cpre, int32_t ldc,
                              void* stream) {
  PCVL_CHECK(A && B && (C || Cb), "null pointer argument");
  PCVL_CHECK(M >= 0 && N >= 0 && K >= 0, "negative GEMM size");
  PCVL_CHECK(epilogue >= 0 && epilogue <= 2, "epilogue must be 0, 1 or 2");
  PCVL_CHECK(epilogue == 0 || bias, "bias epilogue needs a bias");
  PCVL_CHECK(beta == 0.f || C, "beta != 0 needs C");
  if (M == 0 || N == 0) return PCVL_OK;
  GemmArgs g{(const __nv_bfloat16*)A, (const __nv_bfloat16*)B, M, N, K, lda, ldb, ldc, transA, transB, alpha, beta,
             bias, epilogue, C, (__nv_bfloat16*)Cb, Cpre};
  dim3 grid((N + GBN - 1) / GBN, (M + GBM - 1) / GBM);
  PCVL_CHECK(grid.y <= 65535, "M too large for one launch (%d)", M);
  gemm_bf16_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(g);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_mlp_elementwise(int32_t op, const void* x, const void* y, int64_t n, void* out, void* out2,
                                    void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  switch (op) {
    case 0:  // GELU backward: out (f32, may be null), out2 (bf16, may be null)
      k_gelu_backward<<<grid1(n), 256, 0, s>>>((const float*)x, (const float*)y, n, (__nv_bfloat16*)out2,
                                               (float*)out);
      break;
    case 1:  // f32 -> bf16
      k_f32_to_bf16<<<grid1(n), 256, 0, s>>>((const float*)x, n, (__nv_bfloat16*)out);
      break;
    default:
      PCVL_CHECK(false, "unknown elementwise op %d", op);
  }
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_colsum(const float* x, int32_t M, int32_t N, int32_t ld, float* out, void* stream) {
  PCVL_CHECK(x && out, "null pointer argument");
  k_colsum<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>(x, M, N, ld, out);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_softmax_xent(const float* logits, int32_t R, int32_t N, const int32_t* target, float scale,
                                 float* logp_target, float* grad, void* gradb, float* all_logp, void* stream) {
  PCVL_CHECK(logits, "null pointer argument");
  k_softmax_xent<<<(int)(((int64_t)R * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      logits, R, N, target, scale, logp_target, grad, (__nv_bfloat16*)gradb, all_logp);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_bag_embed(const int32_t* seq, int32_t S, int32_t n, int32_t step, const float* mode_emb,
                              const float* pos_emb, int32_t D, void* h, void* stream) {
  PCVL_CHECK(seq && mode_emb && pos_emb && h, "null pointer argument");
  PCVL_CHECK(step < n, "step outside the sequence");
  const int64_t rows = step < 0 ? (int64_t)S * n : S;
  if (rows == 0) return PCVL_OK;
  k_bag_embed<<<(unsigned)rows, 128, 0, (cudaStream_t)stream>>>(seq, S, n, step, mode_emb, pos_emb, D,
                                                                 (__nv_bfloat16*)h);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_bag_embed_backward(const int32_t* seq, int32_t S, int32_t n, const float* dh, int32_t D,
                                       float* dmode, float* dpos, void* stream) {
  PCVL_CHECK(seq && dh && dmode && dpos, "null pointer argument");
  if ((int64_t)S * n == 0) return PCVL_OK;
  k_bag_embed_backward<<<S * n, 128, 0, (cudaStream_t)stream>>>(seq, S, n, dh, D, dmode, dpos);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_adam(float* w, const float* g, float* m1, float* m2, int64_t n, float lr, float b1, float b2,
                         float eps, int32_t step, void* wb, void* stream) {
  PCVL_CHECK(w && g && m1 && m2, "null pointer argument");
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<grid1(n), 256, 0, (cudaStream_t)stream>>>(w, g, m1, m2, n, lr, b1, b2, eps, c1, c2, (__nv_bfloat16*)wb);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_sample_step(const float* logits, int32_t S, int32_t N, int32_t step, uint64_t seed,
                                uint64_t chain0, int32_t* seq, int32_t n, double* logq, void* stream) {
  PCVL_CHECK(logits && seq && logq, "null pointer argument");
  PCVL_CHECK(step >= 0 && step < n, "step outside the sequence");
  k_sample_step<<<(int)(((int64_t)S * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      logits, S, N, step, (uint32_t)seed, (uint32_t)(seed >> 32), chain0, seq, n, logq);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}
