// Glynn / Ryser permanent kernel, one instantiation per matrix size N.
//
// Work split.  The n - 1 free Glynn signs (all n Ryser subset bits) are split into
// L "lo" bits enumerated by every thread's inner loop and H "hi" bits that select
// the thread's pattern.  With the outer sum r_i(hi, lo) = H_i(hi) + T_i(lo), each
// step costs n complex adds (the row sums are rebuilt from two exact-ish parts, so
// no Gray-code drift accumulates) and n - 1 complex multiplies in a balanced tree.
// The table T (2^L x n, in shared memory) is read with warp-broadcast loads.
//
//   Glynn (Glynn 2010):  perm(A) = 2^{1-n} sum_{d in {+-1}^n, d_0 = 1} (prod_k d_k)
//                                   prod_i sum_j d_j a_ij
//   Ryser (Ryser 1963):  perm(A) = (-1)^n sum_{S subset [n]} (-1)^{|S|} prod_i sum_{j in S} a_ij
//
// Bit layout.  Glynn: lo bit l is the sign of column 1 + l, hi bit t the sign of
// column 1 + L + t (bit set = -1).  Ryser: lo bit l includes column l, hi bit t
// column L + t.  Term sign = (-1)^(popc(lo) + popc(hi)) in both.
//
// Work item = (matrix of the bin, chunk of threads * P consecutive hi patterns);
// each CTA writes one FP64 partial sum; pcvl_perm_reduce adds the partials of a
// matrix with compensation and applies the 2^{1-n} (or (-1)^n) and row-scaling
// factors.
#pragma once
#include "common.cuh"

namespace pcvl {

struct PermBinArgs {
  const cdd* A;           // prepared (scaled, df64) matrices
  const int64_t* offs;    // element offset of each matrix in A (global matrix index)
  const int32_t* mids;    // matrix ids of this bin
  int32_t nmat;           // matrices in the bin
  int32_t L;              // lo bits
  int32_t Hbits;          // hi bits
  int64_t P;              // hi patterns per thread per item
  int64_t items_per_mat;  // CTAs per matrix
  int32_t ryser;          // 0 Glynn, 1 Ryser
  double2* partials;      // one per item, bin-local indexing
  cudaStream_t stream;
};

constexpr int kPermThreads = 128;

// prod_i (H_i + T_i) over rows [LO, HI) as a balanced tree.  Glynn uses the lazy
// float-float operations; Ryser, whose alternating subset sum cancels far more, keeps
// every intermediate normalised.
template <int LO, int HI, bool LAZY>
struct RowProd {
  static __device__ __forceinline__ cdd run(const cdd* H, const cdd* Tb) {
    if constexpr (HI - LO == 1) {
      return LAZY ? cdd_add_lazy(H[LO], Tb[LO]) : cdd_add(H[LO], Tb[LO]);
    } else {
      constexpr int MID = (LO + HI) / 2;
      const cdd a = RowProd<LO, MID, LAZY>::run(H, Tb);
      const cdd b = RowProd<MID, HI, LAZY>::run(H, Tb);
      return LAZY ? cdd_mul_lazy(a, b) : cdd_mul(a, b);
    }
  }
};

// signed sum over the lo patterns of one hi pattern
template <int N, bool LAZY>
__device__ __forceinline__ void lo_sweep(const cdd* H, const cdd* T, int nsteps, int hsign, float& arh, float& arl,
                                         float& aih, float& ail) {
  for (int b = 0; b < nsteps; ++b) {
    cdd prod = RowProd<0, N, LAZY>::run(H, T + b * N);
    if ((__popc(b) & 1) ^ hsign) prod = cdd_neg(prod);
    const dd r = two_sum(arh, prod.re.hi);
    const dd i = two_sum(aih, prod.im.hi);
    arh = r.hi;
    arl += r.lo + prod.re.lo;
    aih = i.hi;
    ail += i.lo + prod.im.lo;
  }
}

__device__ __forceinline__ cdd shfl_down_cdd(cdd v, int d) {
  cdd r;
  r.re.hi = __shfl_down_sync(0xffffffffu, v.re.hi, d);
  r.re.lo = __shfl_down_sync(0xffffffffu, v.re.lo, d);
  r.im.hi = __shfl_down_sync(0xffffffffu, v.im.hi, d);
  r.im.lo = __shfl_down_sync(0xffffffffu, v.im.lo, d);
  return r;
}

template <int N>
__global__ void __launch_bounds__(kPermThreads) perm_bin_kernel(PermBinArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cdd* As = reinterpret_cast<cdd*>(smem_raw);  // N x N
  cdd* T = As + N * N;                         // (1 << L) x N
  __shared__ cdd red[kPermThreads / 32];

  const int64_t item = blockIdx.x;
  const int64_t mat_local = item / a.items_per_mat;
  const int64_t chunk = item - mat_local * a.items_per_mat;
  const int mid = a.mids[mat_local];
  const cdd* A = a.A + a.offs[mid];
  const int L = a.L;
  const int ryser = a.ryser;
  const int tid = threadIdx.x;

  for (int e = tid; e < N * N; e += blockDim.x) As[e] = A[e];
  __syncthreads();

  // table: T[b][i] = lo part of row sum i for lo pattern b, built level by level
  const int lo_col0 = ryser ? 0 : 1;
  for (int i = tid; i < N; i += blockDim.x) {
    cdd t0 = cdd_zero();
    if (!ryser)
      for (int l = 0; l < L; ++l) t0 = cdd_add(t0, As[i * N + lo_col0 + l]);
    T[i] = t0;
  }
  __syncthreads();
  for (int l = 0; l < L; ++l) {
    const int half = 1 << l;
    for (int e = tid; e < half * N; e += blockDim.x) {
      const int b = e / N, i = e - b * N;
      cdd d = As[i * N + lo_col0 + l];
      if (!ryser) d = cdd_ldexp(cdd_neg(d), 1);
      T[(b + half) * N + i] = cdd_add(T[b * N + i], d);
    }
    __syncthreads();
  }

  const uint64_t nhi = 1ull << a.Hbits;
  const uint64_t h0 = (uint64_t)chunk * (uint64_t)(kPermThreads * a.P) + (uint64_t)tid * a.P;
  const int hi_col0 = ryser ? L : 1 + L;
  const int nsteps = 1 << L;
  // signed sum of the products: high parts through two_sum, the rest in float
  float arh = 0.f, arl = 0.f, aih = 0.f, ail = 0.f;

  for (int64_t p = 0; p < a.P; ++p) {
    const uint64_t h = h0 + p;
    if (h >= nhi) break;
    cdd H[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      cdd v = ryser ? cdd_zero() : As[i * N];
      for (int t = 0; t < a.Hbits; ++t) {
        const cdd x = As[i * N + hi_col0 + t];
        const bool bit = (h >> t) & 1ull;
        if (ryser) {
          if (bit) v = cdd_add(v, x);
        } else {
          v = cdd_add(v, bit ? cdd_neg(x) : x);
        }
      }
      H[i] = v;
    }
    const int hsign = __popcll(h) & 1;
    if (ryser)
      lo_sweep<N, false>(H, T, nsteps, hsign, arh, arl, aih, ail);
    else
      lo_sweep<N, true>(H, T, nsteps, hsign, arh, arl, aih, ail);
    // fold the low parts in every hi pattern so they stay small
    const dd r = two_sum(arh, arl);
    const dd i = two_sum(aih, ail);
    arh = r.hi;
    arl = r.lo;
    aih = i.hi;
    ail = i.lo;
  }
  cdd acc = {{arh, arl}, {aih, ail}};

  // block reduction (df64), one FP64 partial per CTA
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc = cdd_add(acc, shfl_down_cdd(acc, d));
  if ((tid & 31) == 0) red[tid >> 5] = acc;
  __syncthreads();
  if (tid == 0) {
    cdd s = red[0];
    for (int w = 1; w < kPermThreads / 32; ++w) s = cdd_add(s, red[w]);
    a.partials[item] = make_double2(dd_to_double(s.re), dd_to_double(s.im));
  }
}

// Launch shape of one bin, for callers that build a CUDA graph node instead of launching.
struct PermNode {
  void* func;
  unsigned grid;
  size_t smem;
};

// Launches the bin on a.stream, or (node != nullptr) only fills in its launch shape.
template <int N>
int launch_perm_bin_n(const PermBinArgs& a, PermNode* node) {
  const size_t smem = (size_t)(N * N + (1 << a.L) * N) * sizeof(cdd);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(perm_bin_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  const int64_t items = (int64_t)a.nmat * a.items_per_mat;
  if (node) {
    node->func = reinterpret_cast<void*>(perm_bin_kernel<N>);
    node->grid = (unsigned)items;
    node->smem = smem;
    return 0;
  }
  perm_bin_kernel<N><<<(unsigned)items, kPermThreads, smem, a.stream>>>(a);
  return (int)cudaGetLastError();
}

// Dispatch over the sizes instantiated in one translation unit.
template <int LO, int HI>
int launch_perm_bin_range(int n, const PermBinArgs& a, PermNode* node) {
  if constexpr (LO > HI) {
    return -1;
  } else {
    if (n == LO) return launch_perm_bin_n<LO>(a, node);
    return launch_perm_bin_range<LO + 1, HI>(n, a, node);
  }
}

int launch_perm_bin_1_12(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_13_20(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_21_26(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_27_32(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_33_36(int n, const PermBinArgs& a, PermNode* node);
int launch_perm_bin_37_40(int n, const PermBinArgs& a, PermNode* node);

constexpr int kPermMaxN = 40;

}  // namespace pcvl
