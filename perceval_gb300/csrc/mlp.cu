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
// The GEMM runs on the 5th-generation tensor cores.  Operands whose rows start on
// 16-byte boundaries (either layout) go to gemm_tma_persistent: TMA-loaded 128-byte
// swizzled tiles, one tcgen05.mma issuer, two 128-column FP32 accumulators in tensor
// memory and four epilogue warps per CTA, two CTAs per SM walking the output tiles (see
// its comment below).  Others go to gemm_tc_kernel: one CTA (4 warps) per 128 x 128 tile
// of C with the FP32 accumulator in tensor memory (128 lanes x 128 columns); per 64-wide
// K step the CTA stages the A and B tiles in shared memory in the canonical K-major
// layout without swizzle (8 x 16-byte core matrices; 128 B between core matrices along
// K, 1024 B between 8-row groups), then one thread issues four tcgen05.mma.kind::f16
// (M = 128, N = 128, K = 16) with BF16 inputs and commits them to an mbarrier; three
// stages filled by 16-byte cp.async keep the tiles of steps k + 1 and k + 2 in flight
// while the MMAs of step k run.  Both epilogues read the accumulator with tcgen05.ld
// (warp w owns TMEM lanes 32 (w % 4) .. +31 = rows of the tile) and apply alpha, beta,
// bias and GELU.  Every mbarrier wait is bounded; a CTA whose wait gives up waits
// (bounded) for what it issued, frees its tensor memory and writes NaN to its tiles.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <mutex>

#include "common.cuh"
#include "runtime.cuh"

namespace pcvl {

constexpr int TBM = 128, TBN = 128, TBK = 64;
constexpr int kTcThreads = 128;
constexpr uint32_t kTileBytes = TBM * TBK * 2;  // one bf16 operand tile, 16 KB
constexpr uint32_t kTmemCols = 128;
constexpr int kStages = 3;                       // operand stages in shared memory (96 KB)
constexpr uint32_t kWaitLimit = 1u << 22;        // mbarrier polls before giving up

enum Epilogue { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2 };

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
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

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row r, k) of a 128 x 64 tile in the no-swizzle K-major layout
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
  return (uint32_t)(((r >> 3) * (TBK / 8) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading-dimension byte offset (next
// core matrix along K), stride byte offset (next 8-row group), version 1, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  const uint64_t lbo = 128, sbo = (TBK / 8) * 128;
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// N = 128, M = 128
__device__ __forceinline__ uint32_t umma_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TBN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* gptr) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(gptr) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// one 128 x 64 operand tile into shared memory (element (r, k) of rows [row0, row0 + 128),
// k in [k0, k0 + 64)), zeros outside the matrix.  Rows with k contiguous in memory go by
// 16-byte cp.async (thread t copies row t); transposed operands are gathered by the
// threads (eight rows of one k per 16-byte load, scattered into the rows' core matrices).
__device__ __forceinline__ void stage_tile(const __nv_bfloat16* __restrict__ G, int trans, int ld, int rows, int K,
                                           int row0, int k0, unsigned char* S) {
  const int tid = threadIdx.x;
  const bool aligned = (ld & 7) == 0 && ((reinterpret_cast<uintptr_t>(G) & 15) == 0);
  if (!trans) {
    const int r = tid, gr = row0 + r;
    const uint32_t sbase = smem_u32(S);
#pragma unroll
    for (int kc = 0; kc < TBK / 8; ++kc) {
      const int gk = k0 + kc * 8;
      const uint32_t off = tile_off(r, kc * 8);
      if (gr < rows && gk + 7 < K && aligned) {
        cp_async16(sbase + off, &G[(size_t)gr * ld + gk]);
      } else {
        __nv_bfloat16 v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          v[e] = (gr < rows && gk + e < K) ? G[(size_t)gr * ld + gk + e] : __float2bfloat16(0.f);
        *reinterpret_cast<uint4*>(S + off) = *reinterpret_cast<const uint4*>(v);
      }
    }
  } else {
    for (int c = tid; c < TBM * TBK / 8; c += kTcThreads) {
      const int kk = c >> 4, r = (c & 15) * 8;
      const int gr = row0 + r, gk = k0 + kk;
      __nv_bfloat16 v[8];
      if (gk < K && gr + 7 < rows && aligned) {
        *reinterpret_cast<uint4*>(v) = *reinterpret_cast<const uint4*>(&G[(size_t)gk * ld + gr]);
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e)
          v[e] = (gk < K && gr + e < rows) ? G[(size_t)gk * ld + gr + e] : __float2bfloat16(0.f);
      }
#pragma unroll
      for (int e = 0; e < 8; ++e) *reinterpret_cast<__nv_bfloat16*>(S + tile_off(r + e, kk)) = v[e];
    }
  }
}

// Epilogue of one thread: 32 accumulator columns of one output row, alpha / beta / bias /
// GELU applied, in groups of 4 columns (one 16-byte store per output when aligned).
__device__ __forceinline__ void store_row32(const GemmArgs& g, const uint32_t (&r)[32], int row, int col_base, bool ok,
                                            bool vec) {
#pragma unroll
  for (int i0 = 0; i0 < 32; i0 += 4) {
    const int col0 = col_base + i0;
    if (col0 >= g.N) break;
    const size_t o0 = (size_t)row * g.ldc + col0;
    float v[4], pre[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int col = col0 + e;
      float x = ok ? g.alpha * __uint_as_float(r[i0 + e]) : __int_as_float(0x7fc00000);
      if (col < g.N) {
        if (g.beta != 0.f) x += g.beta * g.C[o0 + e];
        if (g.epi != EPI_NONE) x += g.bias[col];
      }
      pre[e] = x;
      v[e] = g.epi == EPI_BIAS_GELU ? gelu_f(x) : x;
    }
    if (vec && col0 + 3 < g.N) {
      if (g.C) *reinterpret_cast<float4*>(g.C + o0) = make_float4(v[0], v[1], v[2], v[3]);
      if (g.Cpre && g.epi == EPI_BIAS_GELU)
        *reinterpret_cast<float4*>(g.Cpre + o0) = make_float4(pre[0], pre[1], pre[2], pre[3]);
      if (g.Cb) {
        __nv_bfloat162 lo = __floats2bfloat162_rn(v[0], v[1]), hi = __floats2bfloat162_rn(v[2], v[3]);
        uint2 q;
        q.x = *reinterpret_cast<uint32_t*>(&lo);
        q.y = *reinterpret_cast<uint32_t*>(&hi);
        *reinterpret_cast<uint2*>(g.Cb + o0) = q;
      }
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (col0 + e < g.N) {
          if (g.C) g.C[o0 + e] = v[e];
          if (g.Cpre && g.epi == EPI_BIAS_GELU) g.Cpre[o0 + e] = pre[e];
          if (g.Cb) g.Cb[o0 + e] = __float2bfloat16(v[e]);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(kTcThreads) gemm_tc_kernel(GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem[];  // kStages x (A tile, B tile)
  __shared__ __align__(8) uint64_t mbar[kStages];
  __shared__ uint32_t tmem_base_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * TBM, n0 = blockIdx.x * TBN;
  const int nk = (g.K + TBK - 1) / TBK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kStages; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[i])));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base_s;
  const uint32_t idesc = umma_idesc();
  bool ok = true;
  int last = -1;  // last committed K step (uniform over the CTA)

  // step j uses stage j % kStages and completes phase (j / kStages) of mbar[j % kStages]
  auto issue = [&](int j) {
    if (j < nk) {
      unsigned char* As = smem + (j % kStages) * 2 * kTileBytes;
      stage_tile(g.A, g.transA, g.lda, g.M, g.K, m0, j * TBK, As);
      stage_tile(g.B, g.transB, g.ldb, g.N, g.K, n0, j * TBK, As + kTileBytes);
    }
    cp_async_commit();  // one group per step, empty past the end
  };
  for (int j = 0; j < kStages - 1; ++j) issue(j);

  for (int kt = 0; kt < nk && ok; ++kt) {
    const int st = kt % kStages;
    asm volatile("cp.async.wait_group %0;" ::"n"(kStages - 2) : "memory");  // step kt has landed
    // generic-proxy and cp.async writes of the tiles -> visible to the tensor cores
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(smem + st * 2 * kTileBytes), b0 = a0 + kTileBytes;
#pragma unroll
      for (int kk = 0; kk < TBK / 16; ++kk) {
        // K slice kk = core matrices 2kk and 2kk + 1 along K (256 B further per slice)
        const uint64_t ad = umma_desc(a0 + kk * 256), bd = umma_desc(b0 + kk * 256);
        const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&mbar[st]))
                   : "memory");
    }
    last = kt;
    // the next refill reuses the stage of step kt - 1: wait for its MMAs (one pending
    // phase per barrier at any time; the outcome is uniform over the CTA)
    if (kt >= 1) {
      const int j = kt - 1;
      ok = __syncthreads_and(mbar_wait(smem_u32(&mbar[j % kStages]), (j / kStages) & 1));
    }
    if (ok) issue(kt + kStages - 1);
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // every MMA done: the last commit covers all earlier ones of the issuing thread.  This
  // wait runs even after a wait gave up, so no MMA is in flight when the tensor memory is
  // released; a CTA whose waits gave up writes NaN instead of reading the accumulator.
  if (last >= 0)
    ok = __syncthreads_and(mbar_wait(smem_u32(&mbar[last % kStages]), (last / kStages) & 1) && ok);
  asm volatile("tcgen05.fence::after_thread_sync;");

  // epilogue: warp w holds rows 32w..32w+31 of the tile, 32 columns per tcgen05.ld
  const int row = m0 + warp * 32 + lane;
  const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
  for (int c0 = 0; c0 < TBN; c0 += 32) {
    uint32_t r[32];
    if (nk > 0 && ok) {
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr + (uint32_t)c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) r[i] = 0u;
    }
    const bool vec = (g.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(g.C) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(g.Cpre) & 15) == 0 && (reinterpret_cast<uintptr_t>(g.Cb) & 7) == 0;
    if (row < g.M) store_row32(g, r, row, n0 + c0, ok, vec);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// ---------------------------------------------------------------- TMA-fed kernel
// Operands whose rows start on 16-byte boundaries come by TMA (cp.async.bulk.tensor,
// 128-byte swizzle).  A K-major operand tile (k contiguous) uses the 128-byte swizzled
// K-major layout (8 rows x 128 B per swizzle atom, 1024 B between 8-row groups); a K slice
// of 16 elements is 32 B further.
constexpr uint32_t kStageBytes = 2 * kTileBytes;  // A and B tiles of one stage

__device__ __forceinline__ uint64_t umma_desc_sw128(uint32_t saddr) {
  const uint64_t lbo = 16, sbo = 1024;
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// MN-major operand (a transposed A or B: the tile's 128 rows contiguous in memory): two TMA
// boxes of 64 rows (128 B) x 64 k, the second 8 KB after the first.  In the 128-byte swizzled
// MN-major layout a swizzle atom is 64 rows x 8 k (8 lines of 128 B, one line per k); atoms
// adjacent in the row direction are LBO = 8 KB apart (the two boxes), atoms adjacent in k
// SBO = 1024 B apart, so a K slice of 16 elements starts 2048 B further.
constexpr uint32_t kMnBoxBytes = 64 * TBK * 2;  // one 64-row x 64-k box, 8 KB

__device__ __forceinline__ uint64_t umma_desc_sw128_mn(uint32_t saddr) {
  const uint64_t lbo = kMnBoxBytes, sbo = 1024;
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// instruction descriptor with the operands' major-ness (bit 15: A MN-major, bit 16: B)
__device__ __forceinline__ uint32_t umma_idesc_t(bool ta, bool tb) {
  return umma_idesc() | ((ta ? 1u : 0u) << 15) | ((tb ? 1u : 0u) << 16);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(mbar)
      : "memory");
}

// Persistent kernel: two CTAs per SM walk the output tiles t = blockIdx.x,
// blockIdx.x + gridDim.x, ... (tile t = row block t / ntn, column block t % ntn, so
// neighbouring CTAs share their A rows in L2).  Six warps per CTA: warp 0 (one thread)
// issues the TMA loads into a kPStages-deep ring, warp 1 (one thread) the tcgen05.mma into
// one of two 128-column accumulators in tensor memory, and warps 2..5 read an accumulator
// back (warp w reads TMEM lanes 32 (w % 4) .. +31), release it, and store it while the MMAs
// of the next tile run into the other one.  The ring and the accumulators are handed over
// by mbarriers: full / empty per stage, acc_full (MMA commit) and acc_empty (the four
// epilogue warps) per accumulator.  Transposed operands (TA / TB) arrive MN-major.
// Measured on GB300 (CUDA-graph replay of back-to-back calls): two CTAs of 3 stages per SM
// beat one CTA of 4, 5 or 6 stages at every shape (8192^3: 1326 against 1036 TFLOP/s), and
// staging the outputs in shared memory for TMA stores was slower than the warps' own
// 16-byte stores.  Every wait is bounded; after one gives up the CTA stops issuing, waits
// (bounded) for the loads and MMAs it issued, and writes NaN to the tiles it had not finished.
constexpr int kPStages = 3;    // 96 KB of operand stages per CTA
constexpr int kPCtasPerSm = 2;  // two CTAs per SM: two load / MMA pipelines and 8 epilogue warps
constexpr uint32_t kPSmemBytes = kPStages * kStageBytes + 1024;
constexpr int kPThreads = 192;
constexpr uint32_t kPTmemCols = 256;

template <bool TA, bool TB>
__global__ void __launch_bounds__(kPThreads, kPCtasPerSm)
    gemm_tma_persistent(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, GemmArgs g,
                        int ntn, int ntiles) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kPStages], empty[kPStages], accf[2], acce[2], done;
  __shared__ uint32_t tmem_base_s;
  __shared__ volatile int fail;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nk = (g.K + TBK - 1) / TBK;
  const uint32_t sbase = (smem_u32(smem_raw) + 1023u) & ~1023u;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                 "r"(kPTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kPStages; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[i])));
    }
    for (int i = 0; i < 2; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&accf[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(smem_u32(&acce[i])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base_s;

  if (warp == 0) {
    if (lane == 0 && nk > 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
      // producer: global step it -> stage it % S, phase it / S of full[] and empty[]
      int it = 0;
      for (int t = blockIdx.x; t < ntiles && !fail; t += gridDim.x) {
        const int m0 = (t / ntn) * TBM, n0 = (t % ntn) * TBN;
        for (int kt = 0; kt < nk; ++kt, ++it) {
          const int st = it % kPStages, round = it / kPStages;
          if (it >= kPStages && !mbar_wait(smem_u32(&empty[st]), (round - 1) & 1)) {
            fail = 1;
            break;
          }
          if (fail) break;
          const uint32_t fb = smem_u32(&full[st]);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(kStageBytes)
                       : "memory");
          const uint32_t a_dst = sbase + st * kStageBytes, b_dst = a_dst + kTileBytes;
          if (TA) {
            tma_load_2d(a_dst, &mapA, m0, kt * TBK, fb);
            tma_load_2d(a_dst + kMnBoxBytes, &mapA, m0 + 64, kt * TBK, fb);
          } else {
            tma_load_2d(a_dst, &mapA, kt * TBK, m0, fb);
          }
          if (TB) {
            tma_load_2d(b_dst, &mapB, n0, kt * TBK, fb);
            tma_load_2d(b_dst + kMnBoxBytes, &mapB, n0 + 64, kt * TBK, fb);
          } else {
            tma_load_2d(b_dst, &mapB, kt * TBK, n0, fb);
          }
        }
      }
      // the last load into each stage has landed before the CTA moves on
      for (int q = (it > kPStages ? it - kPStages : 0); q < it; ++q)
        if (!mbar_wait(smem_u32(&full[q % kPStages]), (q / kPStages) & 1)) fail = 1;
    }
  } else if (warp == 1) {
    if (lane == 0 && nk > 0) {
      const uint32_t idesc = umma_idesc_t(TA, TB);
      int it = 0, lt = 0;
      for (int t = blockIdx.x; t < ntiles && !fail; t += gridDim.x, ++lt) {
        const int buf = lt & 1, use = lt >> 1;
        if (lt >= 2 && !mbar_wait(smem_u32(&acce[buf]), (use - 1) & 1)) {
          fail = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t acc_addr = tmem + (uint32_t)(buf * TBN);
        bool stop = false;
        for (int kt = 0; kt < nk; ++kt, ++it) {
          const int st = it % kPStages;
          if (!mbar_wait(smem_u32(&full[st]), (it / kPStages) & 1)) {
            fail = 1;
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t a0 = sbase + st * kStageBytes, b0 = a0 + kTileBytes;
#pragma unroll
          for (int kk = 0; kk < TBK / 16; ++kk) {
            const uint64_t ad = TA ? umma_desc_sw128_mn(a0 + kk * 2048) : umma_desc_sw128(a0 + kk * 32);
            const uint64_t bd = TB ? umma_desc_sw128_mn(b0 + kk * 2048) : umma_desc_sw128(b0 + kk * 32);
            const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc_addr),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&empty[st]))
                       : "memory");
        }
        if (stop) break;
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&accf[buf]))
                     : "memory");
      }
      // every MMA issued has completed before tensor memory is released
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&done))
                   : "memory");
      if (!mbar_wait(smem_u32(&done), 0)) fail = 1;
    }
  } else {
    // epilogue warps 2..5: warp w owns the accumulator rows 32 (w % 4) .. +31
    const int quad = warp & 3;
    const bool vec = (g.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(g.C) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(g.Cpre) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(g.Cb) & 7) == 0;
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      const int m0 = (t / ntn) * TBM, n0 = (t % ntn) * TBN;
      const int buf = lt & 1, use = lt >> 1;
      bool ok = nk > 0 && !fail;
      if (ok && !mbar_wait(smem_u32(&accf[buf]), use & 1)) {
        fail = 1;
        ok = false;
      }
      ok = __all_sync(0xffffffffu, ok);
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int row = m0 + quad * 32 + lane;
      const uint32_t taddr = tmem + (uint32_t)(buf * TBN) + ((uint32_t)(quad * 32) << 16);
#pragma unroll 1
      for (int c0 = 0; c0 < TBN; c0 += 32) {
        uint32_t r[32];
        if (ok) {
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
              "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
              : "r"(taddr + (uint32_t)c0));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) r[i] = 0u;
        }
        if (c0 + 32 >= TBN) {
          // the accumulator is in registers: the MMAs of tile lt + 2 may start
          asm volatile("tcgen05.fence::before_thread_sync;");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acce[buf])) : "memory");
        }
        if (row < g.M) store_row32(g, r, row, n0 + c0, ok, vec);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPTmemCols));
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

// Tensor map of a row-major bf16 matrix (rows x k, row stride ld elements) for 128-row x
// 64-element boxes with the 128-byte swizzle; out-of-range elements read as zero.
// Tensor map of one operand: K-major (rows x k, k contiguous; box 64 k x 128 rows) or, for a
// transposed operand, MN-major (k x rows, rows contiguous; box 64 rows x 64 k).
enum MapKind { kMapK = 0, kMapMN = 1 };

static int make_tile_map(CUtensorMap* map, const void* base, int k, int rows, int ld, int kind) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    PCVL_CHECK(e == cudaSuccess && q == cudaDriverEntryPointSuccess && fn, "cuTensorMapEncodeTiled is unavailable");
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const bool mn = kind == kMapMN;
  const cuuint64_t dims[2] = {(cuuint64_t)(mn ? rows : k), (cuuint64_t)(mn ? k : rows)};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {mn ? 64u : (cuuint32_t)TBK, mn ? (cuuint32_t)TBK : (cuuint32_t)TBM};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  PCVL_CHECK(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return PCVL_OK;
}

static int grid1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 65536)); }

// The training loop calls the same few GEMM shapes on the same buffers every step: tensor
// maps are kept in a small table keyed by (device, base, k, rows, ld) instead of encoded per
// call, and each kernel's shared-memory limit is raised once per device.
struct MapKey {
  int dev;
  const void* base;
  int k, rows, ld, kind;
};
struct MapEntry {
  MapKey key;
  CUtensorMap map;
};
static MapEntry g_maps[64];
static int g_nmaps = 0, g_next_map = 0;
static std::mutex g_maps_mu;

static int cached_tile_map(CUtensorMap* map, const void* base, int k, int rows, int ld, int kind) {
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_maps_mu);
  for (int i = 0; i < g_nmaps; ++i) {
    const MapKey& q = g_maps[i].key;
    if (q.dev == dev && q.base == base && q.k == k && q.rows == rows && q.ld == ld && q.kind == kind) {
      *map = g_maps[i].map;
      return PCVL_OK;
    }
  }
  PCVL_TRY(make_tile_map(map, base, k, rows, ld, kind));
  MapEntry& e = g_maps[g_next_map];
  e.key = {dev, base, k, rows, ld, kind};
  e.map = *map;
  g_next_map = (g_next_map + 1) % 64;
  g_nmaps = std::min(g_nmaps + 1, 64);
  return PCVL_OK;
}

// Raises a kernel's dynamic shared-memory limit once per (device, kernel): the GEMM has five
// kernels (four operand layouts of the persistent one and the cp.async one).
static int allow_smem(const void* func, int bytes) {
  constexpr int kSlots = 8;
  static std::mutex mu;
  static const void* done_func[64][kSlots] = {};
  static int done_bytes[64][kSlots] = {};
  int dev = 0;
  PCVL_CUDA(cudaGetDevice(&dev));
  PCVL_CHECK(dev >= 0 && dev < 64, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  int slot = -1;
  for (int i = 0; i < kSlots; ++i) {
    if (done_func[dev][i] == func) {
      if (done_bytes[dev][i] >= bytes) return PCVL_OK;
      slot = i;
      break;
    }
    if (slot < 0 && done_func[dev][i] == nullptr) slot = i;
  }
  PCVL_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  if (slot >= 0) {
    done_func[dev][slot] = func;
    done_bytes[dev][slot] = bytes;
  }
  return PCVL_OK;
}

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
  dim3 grid((N + TBN - 1) / TBN, (M + TBM - 1) / TBM);
  PCVL_CHECK(grid.y <= 65535, "M too large for one launch (%d)", M);
  // rows (of either layout) 16-byte aligned: TMA-fed persistent kernel; anything else: cp.async
  const bool tma = K > 0 && (lda % 8) == 0 && (ldb % 8) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(B) & 15) == 0;
  if (tma) {
    CUtensorMap mapA, mapB;
    PCVL_TRY(cached_tile_map(&mapA, A, K, M, lda, transA ? kMapMN : kMapK));
    PCVL_TRY(cached_tile_map(&mapB, B, K, N, ldb, transB ? kMapMN : kMapK));
    // persistent: two CTAs per SM over every tile of the output
    const int ntiles = (int)grid.x * (int)grid.y;
    const int ctas = std::min(ntiles, kPCtasPerSm * num_sms());
    const int smem = (int)kPSmemBytes;
    void (*kern)(const CUtensorMap, const CUtensorMap, GemmArgs, int, int) =
        transA ? (transB ? gemm_tma_persistent<true, true> : gemm_tma_persistent<true, false>)
               : (transB ? gemm_tma_persistent<false, true> : gemm_tma_persistent<false, false>);
    PCVL_TRY(allow_smem(reinterpret_cast<const void*>(kern), smem));
    kern<<<ctas, kPThreads, smem, (cudaStream_t)stream>>>(mapA, mapB, g, (int)grid.x, ntiles);
  } else {
    const int smem = kStages * 2 * (int)kTileBytes;
    PCVL_TRY(allow_smem(reinterpret_cast<const void*>(gemm_tc_kernel), smem));
    gemm_tc_kernel<<<grid, kTcThreads, smem, (cudaStream_t)stream>>>(g);
  }
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
