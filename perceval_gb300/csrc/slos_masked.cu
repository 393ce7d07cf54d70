// Masked SLOS: the layer chain restricted to the Fock states a mask can still accept.
//
// Semantics (perceval/backends/_abstract_backends.py:103-137, _slos.py:152-166).  A mask
// is a list of strings with one character per mode.  A digit fixes that mode's photon
// count; a space or '*' accepts any count; a mode listed in at_least_modes accepts any
// count >= its digit.  A state is accepted when it matches one of the strings.  The
// reference restricts every layer k with the same mask (xq.FSArray(m, k, mask),
// _slos.py:161-164): layer k keeps the k-photon states that can still be completed to an
// accepted state of N photons (N = the mask's photon count).  For one string that means
// v_i <= d_i on every fixed mode, and the photons still missing,
// sum over constrained modes of max(d_i - v_i, 0), are at most N - k.  The outputs are
// the kept states of layer n, in descending lexicographic order (allstate_iterator with
// a mask, perceval/utils/states.py:268-290).
//
// Closure.  If c is kept, every parent c - e_j is kept: removing a photon keeps
// v_i <= d_i, and the missing count grows by at most one while N - k grows by one.  So
// the gather
//     c_k[c] = sum_{j : c_j > 0} u_j c_{k-1}[c - e_j]
// over kept parents is exact: the kept amplitudes equal those of the full space.
//
// Building the kept sets without enumerating the full space.  A state c of k photons
// has one canonical parent p = c - e_l (l: its last occupied mode), and c = p + e_j
// with j >= the last occupied mode of p.  Generating, for the kept states p of layer
// k-1 in order, the accepted children p + e_j for j = last(p) .. m-1 therefore visits
// every kept state of layer k exactly once, and in descending lexicographic order.
// For p before p', let i be the first mode where they differ: p_i > p'_i, and p' has
// photons after mode i, so every child of p' holds fewer photons at i than every
// child of p.  Kept states are stored as their ranks in the full k-photon space
// (ascending rank = descending lexicographic order).  The parent index of state c
// through mode j is the position of rank(c - e_j) in the previous layer's list (binary
// search, at plan creation).  The kernels then read per state one occupied-mode bit
// mask and one parent index per occupied mode.
//
// Ranks (the full space, as in slos.cu): with Cn(M, x) = C(M + x - 1, x) and R_{i+1}
// the photons in modes after i,
//     rank(s)       = sum_{i <= m-2} Cn(m - i, R_{i+1} - 1)
//     rank(p + e_j) = rank(p) + sum_{i < j} Cn(m - i - 1, R_{i+1}(p)).
//
// Arithmetic: the kernels are instantiated for the two policies of arith.cuh (FP64, the
// default, and float-float), as the full-space kernels of slos.cu.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "arith.cuh"
#include "common.cuh"
#include "runtime.cuh"
#include "slos_plan.cuh"

namespace pcvl {
namespace {

constexpr int kMaskMaxM = 32;
constexpr int kMaskMaxN = 32;
constexpr int kMaxMasks = 64;
constexpr uint32_t kNoIdx = 0xffffffffu;
constexpr int kGenThreads = 256;

struct MaskSpace {
  int m, N, nmask;
  uint32_t at_least;      // modes whose digit is a lower bound
  int cs;                 // row stride of cn
  const int8_t* digits;   // [nmask][m]; -1: any count
  const uint64_t* cn;     // cn[M * cs + x] = Cn(M, x), M = 0..m, x = 0..cs-1
};

__device__ __forceinline__ uint64_t cnv(const MaskSpace& s, int M, int x) {
  return x < 0 ? 0ull : s.cn[M * s.cs + x];
}

// The table Cn in shared memory for the kernels that unrank every state: returns the
// space with cn pointing to the shared copy.
constexpr int kCnWords = (kMaskMaxM + 1) * (kMaskMaxN + 2);
__device__ __forceinline__ MaskSpace shared_cn(const MaskSpace& s, uint64_t* buf) {
  const int words = (s.m + 1) * s.cs;
  for (int i = threadIdx.x; i < words; i += blockDim.x) buf[i] = s.cn[i];
  __syncthreads();
  MaskSpace t = s;
  t.cn = buf;
  return t;
}

// Occupation of the state of rank r among the k-photon states.  On modes i..m-1 with
// rem photons, the states with R_{i+1} = y photons after mode i number Cn(m-i-1, y)
// and come in increasing y; their cumulative count up to y = x is Cn(m - i, x).
__device__ void unrank_state(const MaskSpace& s, int k, uint64_t r, uint8_t* v) {
  int rem = k;
  for (int i = 0; i < s.m - 1; ++i) {
    int x = 0;
    while (x < rem && r >= cnv(s, s.m - i, x)) ++x;
    r -= cnv(s, s.m - i, x - 1);
    v[i] = (uint8_t)(rem - x);
    rem = x;
  }
  v[s.m - 1] = (uint8_t)rem;
}

// Bit j set when the child p + e_j (j >= lo) of the (k-1)-photon state v is kept in layer k.
__device__ uint32_t accepted_children(const MaskSpace& s, int k, const uint8_t* v, int lo) {
  uint32_t ok = 0;
  const int spare = s.N - k;
  for (int q = 0; q < s.nmask; ++q) {
    const int8_t* dg = s.digits + (size_t)q * s.m;
    int miss = 0;
    bool fail = false;
    for (int i = 0; i < s.m; ++i) {
      const int d = dg[i];
      if (d < 0) continue;
      const int vi = v[i];
      if ((s.at_least >> i) & 1u) {
        if (vi < d) miss += d - vi;
      } else if (vi > d) {
        fail = true;
        break;
      } else {
        miss += d - vi;
      }
    }
    if (fail) continue;
    for (int j = lo; j < s.m; ++j) {
      const int d = dg[j];
      int mj = miss;
      if (d >= 0) {
        if ((s.at_least >> j) & 1u) {
          if (v[j] < d) --mj;
        } else if (v[j] + 1 > d) {
          continue;
        } else {
          --mj;
        }
      }
      if (mj <= spare) ok |= 1u << j;
    }
  }
  return ok;
}

// Kept states of layer k from those of layer k-1 (one thread per parent; block b owns
// parents b * 256 ..).  Count pass (out == nullptr): the block's number of kept
// children to bsum[b].  Write pass: their full-space ranks, in parent order then mode
// order, from position boff[b].
__global__ void __launch_bounds__(kGenThreads) mask_gen(MaskSpace sg, int k, const uint64_t* __restrict__ prev,
                                                       uint64_t nprev, const uint64_t* __restrict__ boff,
                                                       uint32_t* __restrict__ bsum, uint64_t* __restrict__ out) {
  __shared__ uint32_t wsum[kGenThreads / 32];
  __shared__ uint64_t cn_s[kCnWords];
  const MaskSpace s = shared_cn(sg, cn_s);
  const uint64_t i = (uint64_t)blockIdx.x * kGenThreads + threadIdx.x;
  uint8_t v[kMaskMaxM];
  uint32_t ok = 0;
  uint64_t r = 0;
  if (i < nprev) {
    r = prev[i];
    unrank_state(s, k - 1, r, v);
    int lo = 0;
    for (int j = s.m - 1; j > 0; --j)
      if (v[j]) {
        lo = j;
        break;
      }
    ok = accepted_children(s, k, v, lo);
  }
  const uint32_t c = __popc(ok);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += t;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  uint32_t wbase = 0, total = 0;
  for (int q = 0; q < kGenThreads / 32; ++q) {
    if (q < w) wbase += wsum[q];
    total += wsum[q];
  }
  if (out == nullptr) {
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
    return;
  }
  if (!ok) return;
  uint64_t pos = boff[blockIdx.x] + wbase + inc - c;
  uint64_t add = 0;  // sum_{i<j} Cn(m - i - 1, R_{i+1}(p))
  int after = k - 1;
  for (int j = 0; j < s.m; ++j) {
    if ((ok >> j) & 1u) out[pos++] = r + add;
    after -= v[j];
    add += cnv(s, s.m - j - 1, after);
  }
}

// Smallest index >= start of a value >= r in the ascending prev[0..n) (n if none):
// exponential probing from start, then a binary search in the bracket.
__device__ __forceinline__ uint64_t gallop(const uint64_t* __restrict__ prev, uint64_t n, uint64_t start,
                                           uint64_t r) {
  uint64_t lo = start, hi = n, step = 1;
  while (true) {
    const uint64_t probe = lo + step - 1;
    if (probe >= n) break;
    if (prev[probe] >= r) {
      hi = probe;
      break;
    }
    lo = probe + 1;
    step <<= 1;
  }
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (prev[mid] < r)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

constexpr int kParentRun = 16;  // most consecutive kept states per thread of mask_parents

// Per kept state i of layer k: occupied-mode bits, the index in layer k-1 of each parent
// (par[e * ncur + i] for its e-th occupied mode) and, on the last layer, prod(out!).
// rank(c - e_j) = rank(c) - sum_{i<j} Cn(m - i - 1, R_{i+1}(c) - 1).  For a fixed mode j,
// c -> c - e_j keeps the order, so a thread takes `run` consecutive states (1 .. kParentRun,
// fewer on small layers to keep every SM busy) and finds each parent by galloping forward
// from the previous state's parent through the same mode.
__global__ void __launch_bounds__(256) mask_parents(MaskSpace sg, int k, const uint64_t* __restrict__ cur,
                                                    uint64_t ncur, const uint64_t* __restrict__ prev,
                                                    uint64_t nprev, uint32_t* __restrict__ occ,
                                                    uint32_t* __restrict__ par, void* __restrict__ fact,
                                                    int fact_f64, int* __restrict__ err, int run_len) {
  __shared__ uint64_t cn_s[kCnWords];
  const MaskSpace s = shared_cn(sg, cn_s);
  const uint64_t runs = (ncur + run_len - 1) / run_len;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t run = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; run < runs; run += stride) {
    uint64_t next[kMaskMaxM];  // per mode: where the next parent search starts
    for (int j = 0; j < s.m; ++j) next[j] = 0;
    const uint64_t i1 = min(ncur, (run + 1) * run_len);
    for (uint64_t i = run * run_len; i < i1; ++i) {
      uint8_t v[kMaskMaxM];
      const uint64_t rc = cur[i];
      unrank_state(s, k, rc, v);
      uint32_t om = 0;
      uint64_t e = 0, sub = 0;
      int after = k;
      double f = 1.0;
      for (int j = 0; j < s.m; ++j) {
        if (v[j]) {
          om |= 1u << j;
          for (int t = 2; t <= v[j]; ++t) f *= (double)t;
          const uint64_t r = rc - sub;
          const uint64_t lo = gallop(prev, nprev, next[j], r);
          uint32_t idx = (uint32_t)lo;
          if (lo >= nprev || prev[lo] != r) {
            atomicExch(err, 1);
            idx = 0;
          } else {
            next[j] = lo + 1;
          }
          par[e * ncur + i] = idx;
          ++e;
        }
        after -= v[j];
        sub += cnv(s, s.m - j - 1, after - 1);
      }
      occ[i] = om;
      if (fact) {
        if (fact_f64)
          static_cast<double*>(fact)[i] = f;
        else
          static_cast<dd*>(fact)[i] = dd_from_double(f);
      }
    }
  }
}

// child[j * nprev + p] = i for every kept state i of layer k with parent p through mode j
// (entries left at kNoIdx: the child is not kept)
__global__ void __launch_bounds__(256) mask_children(const uint32_t* __restrict__ occ,
                                                     const uint32_t* __restrict__ par, uint64_t ncur,
                                                     uint64_t nprev, uint32_t* __restrict__ child) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncur; i += stride) {
    uint64_t e = i;
    for (uint32_t om = occ[i]; om; om &= om - 1, e += ncur) {
      const int j = __ffs(om) - 1;
      child[(uint64_t)j * nprev + par[e]] = (uint32_t)i;
    }
  }
}

// u_j (conjugated for the adjoint) of one circuit, or of the CTA's 32 circuits as [j][lane]
template <bool BATCHED, bool CONJ, class P>
__device__ __forceinline__ void load_u(typename P::V* us, const typename P::V* __restrict__ ucol, int m, int B) {
  using V = typename P::V;
  if (BATCHED) {
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
      const int j = t >> 5, b = blockIdx.y * 32 + (t & 31);
      const V v = (j < m && b < B) ? ucol[(size_t)j * B + b] : P::zero();
      us[t] = CONJ ? P::conj(v) : v;
    }
  } else if (threadIdx.x < 32) {
    const V v = (int)threadIdx.x < m ? ucol[threadIdx.x] : P::zero();
    us[threadIdx.x] = CONJ ? P::conj(v) : v;
  }
  __syncthreads();
}

// Layer k: c_k[i] = sum_e u_{j_e} c_{k-1}[par[e][i]] over the occupied modes j_e of kept
// state i.  One thread per state (one circuit) or one warp per state with the lanes
// over 32 circuits (blockIdx.y selects the chunk).
template <bool BATCHED, class P>
__global__ void __launch_bounds__(256) slos_mfwd(const typename P::V* __restrict__ in, typename P::V* __restrict__ out,
                                                 const uint32_t* __restrict__ occ,
                                                 const uint32_t* __restrict__ par, uint64_t L,
                                                 const typename P::V* __restrict__ ucol, int m, int B) {
  using V = typename P::V;
  __shared__ V us[BATCHED ? 32 * 32 : 32];
  load_u<BATCHED, false, P>(us, ucol, m, B);
  if (!BATCHED) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += stride) {
      typename P::Acc acc = P::acc_zero();
      uint64_t e = i;
      for (uint32_t om = __ldg(&occ[i]); om; om &= om - 1, e += L)
        P::fma(acc, P::ld(&in[__ldg(&par[e])]), us[__ffs(om) - 1]);
      out[i] = P::finish(acc);
    }
  } else {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.y * 32 + lane;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t i = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < L; i += nw) {
      typename P::Acc acc = P::acc_zero();
      uint64_t e = i;
      for (uint32_t om = __ldg(&occ[i]); om; om &= om - 1, e += L) {
        const uint32_t pidx = __ldg(&par[e]);
        if (b < B) P::fma(acc, P::ld(&in[(size_t)pidx * B + b]), us[(__ffs(om) - 1) * 32 + lane]);
      }
      if (b < B) out[i * B + b] = P::finish(acc);
    }
  }
}

// Kept outputs -> probabilities (mode 0), amplitudes (mode 1) or the adjoint seed
// a_n = 2 w F c_n (mode 2), with F = prod(out!) / prod(in_b!).
template <class P>
__global__ void __launch_bounds__(256) slos_mfin(const typename P::V* __restrict__ c,
                                                 const typename P::F* __restrict__ fact,
                                                 const typename P::F* __restrict__ inv_in, uint64_t L, int B,
                                                 int mode, const double* __restrict__ w,
                                                 double* __restrict__ out_real, double2* __restrict__ out_c,
                                                 typename P::V* __restrict__ seed) {
  const uint64_t tot = L * (uint64_t)B;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < tot; idx += stride) {
    const uint64_t i = idx / (uint64_t)B;
    const int b = (int)(idx - i * (uint64_t)B);
    const typename P::F F = P::f_mul(fact[i], inv_in[b]);
    const typename P::V v = P::ld(&c[idx]);
    if (mode == 0)
      out_real[idx] = P::prob(v, F);
    else if (mode == 1)
      out_c[idx] = P::amp(v, F);
    else
      seed[idx] = P::seed(v, w[idx], F);
  }
}

// Adjoint step over the kept states of layer k-1: a_{k-1}[i] = sum_j conj(u_j) a_k[child_j(i)]
// and g_j += conj(c_{k-1}[i]) a_k[child_j(i)] over the kept children; per-CTA partials of
// g to gpart[cta][j][b].
template <int MMAX, bool BATCHED, class P>
__global__ void __launch_bounds__(256) slos_mbwd(const typename P::V* __restrict__ ain,
                                                 typename P::V* __restrict__ aout,
                                                 const typename P::V* __restrict__ cpar,
                                                 const uint32_t* __restrict__ child, uint64_t Lp,
                                                 const typename P::V* __restrict__ ucol, int m, int B,
                                                 typename P::V* __restrict__ gpart) {
  using V = typename P::V;
  __shared__ V us[BATCHED ? 32 * 32 : 32];
  __shared__ V red[8][32];
  load_u<BATCHED, true, P>(us, ucol, m, B);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int b = BATCHED ? blockIdx.y * 32 + lane : 0;
  typename P::Acc g[MMAX];
#pragma unroll
  for (int j = 0; j < MMAX; ++j) g[j] = P::acc_zero();
  const uint64_t per = BATCHED ? (blockDim.x >> 5) : blockDim.x;
  const uint64_t first = (uint64_t)blockIdx.x * per + (BATCHED ? wid : threadIdx.x);
  const uint64_t stride = (uint64_t)gridDim.x * per;
  for (uint64_t i = first; i < Lp; i += stride) {
    if (BATCHED && b >= B) continue;
    const size_t pidx = BATCHED ? (size_t)i * B + b : (size_t)i;
    const V cp = P::conj(P::ld(&cpar[pidx]));
    typename P::Acc acc = P::acc_zero();
#pragma unroll
    for (int j = 0; j < MMAX; ++j) {
      if (j < m) {
        const uint32_t ci = __ldg(&child[(uint64_t)j * Lp + i]);
        if (ci != kNoIdx) {
          const V v = P::ld(&ain[BATCHED ? (size_t)ci * B + b : (size_t)ci]);
          P::fma(acc, v, us[BATCHED ? j * 32 + lane : j]);
          P::fma(g[j], v, cp);
        }
      }
    }
    aout[pidx] = P::finish(acc);
  }
#pragma unroll
  for (int j = 0; j < MMAX; ++j) {
    if (j >= m) break;
    V v = P::finish(g[j]);
    if (!BATCHED) {
#pragma unroll
      for (int dlt = 16; dlt > 0; dlt >>= 1) v = P::add(v, P::shfl_down(v, dlt));
    }
    red[wid][lane] = v;
    __syncthreads();
    if (wid == 0) {
      if (BATCHED) {
        V s2 = red[0][lane];
        for (int q = 1; q < 8; ++q) s2 = P::add(s2, red[q][lane]);
        if (b < B) gpart[((size_t)blockIdx.x * m + j) * B + b] = s2;
      } else if (lane == 0) {
        V s2 = red[0][0];
        for (int q = 1; q < 8; ++q) s2 = P::add(s2, red[q][0]);
        gpart[(size_t)blockIdx.x * m + j] = s2;
      }
    }
    __syncthreads();
  }
}

// grad[b][j][col[b]] += sum over CTAs of gpart[cta][j][b]
template <class P>
__global__ void slos_mgrad_reduce(const typename P::V* __restrict__ gpart, int nblk, int m, int B,
                                  const int32_t* __restrict__ col, double2* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * B) return;
  const int j = i / B, b = i - j * B;
  typename P::V s = P::zero();
  for (int q = 0; q < nblk; ++q) s = P::add(s, gpart[(size_t)q * m * B + i]);
  double2* g = &grad[((size_t)b * m + j) * m + col[b]];
  g->x += P::re(s);
  g->y += P::im(s);
}

// device buffer released at scope exit unless taken
struct TmpBuf {
  void* p = nullptr;
  ~TmpBuf() { cudaFree(p); }
  void* take() {
    void* q = p;
    p = nullptr;
    return q;
  }
};

int tmp_alloc(TmpBuf& b, size_t bytes) {
  if (cudaMalloc(&b.p, bytes < 256 ? 256 : bytes) != cudaSuccess) {
    b.p = nullptr;
    set_error("masked SLOS plan: device allocation of %zu bytes failed", bytes);
    return PCVL_ERR_MEMORY;
  }
  return PCVL_OK;
}

int grid_for(uint64_t threads, int per_sm) {
  const uint64_t g = std::min<uint64_t>((threads + 255) / 256, (uint64_t)num_sms() * per_sm);
  return (int)std::max<uint64_t>(g, 1);
}

template <int MMAX, class P>
void launch_mbwd(bool batched, dim3 grid, const void* ain, void* aout, const void* cpar, const uint32_t* child,
                 uint64_t Lp, const void* ucol, int m, int B, void* gpart, cudaStream_t s) {
  using V = typename P::V;
  if (batched)
    slos_mbwd<MMAX, true, P><<<grid, 256, 0, s>>>((const V*)ain, (V*)aout, (const V*)cpar, child, Lp,
                                                  (const V*)ucol, m, B, (V*)gpart);
  else
    slos_mbwd<MMAX, false, P><<<grid, 256, 0, s>>>((const V*)ain, (V*)aout, (const V*)cpar, child, Lp,
                                                   (const V*)ucol, m, B, (V*)gpart);
}

template <class P>
void launch_mbwd_m(bool batched, dim3 grid, const void* ain, void* aout, const void* cpar, const uint32_t* child,
                   uint64_t Lp, const void* ucol, int m, int B, void* gpart, cudaStream_t s) {
  if (m <= 8)
    launch_mbwd<8, P>(batched, grid, ain, aout, cpar, child, Lp, ucol, m, B, gpart, s);
  else if (m <= 16)
    launch_mbwd<16, P>(batched, grid, ain, aout, cpar, child, Lp, ucol, m, B, gpart, s);
  else if (m <= 24)
    launch_mbwd<24, P>(batched, grid, ain, aout, cpar, child, Lp, ucol, m, B, gpart, s);
  else
    launch_mbwd<32, P>(batched, grid, ain, aout, cpar, child, Lp, ucol, m, B, gpart, s);
}

}  // namespace

void slos_masked_free(pcvl_slos_plan* p) {
  for (uint32_t* q : p->mocc_d) cudaFree(q);
  for (uint32_t* q : p->mpar_d) cudaFree(q);
  for (uint32_t* q : p->mchild_d) cudaFree(q);
  cudaFree(p->mrank_d);
  cudaFree(p->mfact_d);
  p->mocc_d.clear();
  p->mpar_d.clear();
  p->mchild_d.clear();
  p->mrank_d = nullptr;
  p->mfact_d = nullptr;
}

int slos_masked_create(pcvl_slos_plan** plan, int32_t m, const int32_t* inputs, int32_t batch,
                       int32_t keep_layers, int32_t n_masks, const int8_t* digits, uint32_t at_least,
                       int32_t mask_n, int32_t precision) {
  PCVL_CHECK(plan && inputs && digits, "null pointer argument");
  *plan = nullptr;
  PCVL_CHECK(precision == kPrecFP64 || precision == kPrecFloatFloat,
             "precision must be %d (FP64) or %d (float-float), got %d", (int)kPrecFP64, (int)kPrecFloatFloat,
             precision);
  PCVL_CHECK(m >= 1 && m <= kMaskMaxM, "m=%d outside [1, %d]", m, kMaskMaxM);
  PCVL_CHECK(batch >= 1, "batch must be >= 1");
  PCVL_CHECK(n_masks >= 1 && n_masks <= kMaxMasks, "n_masks=%d outside [1, %d]", n_masks, kMaxMasks);
  PCVL_CHECK(mask_n >= 0, "mask photon count %d is negative", mask_n);
  for (int q = 0; q < n_masks * m; ++q)
    PCVL_CHECK(digits[q] >= -1, "mask digit %d at position %d: digits are counts >= 0, or -1 for any", digits[q], q);
  int n = -1;
  for (int b = 0; b < batch; ++b) {
    int nb = 0;
    for (int i = 0; i < m; ++i) {
      PCVL_CHECK(inputs[(size_t)b * m + i] >= 0, "negative photon count in input state %d", b);
      nb += inputs[(size_t)b * m + i];
    }
    PCVL_CHECK(n < 0 || nb == n, "input state %d has %d photons, state 0 has %d: a plan needs one photon count", b,
               nb, n);
    n = nb;
  }
  PCVL_CHECK(n <= kMaskMaxN, "n=%d photons exceeds %d", n, kMaskMaxN);

  auto* p = new (std::nothrow) pcvl_slos_plan();
  PCVL_CHECK(p, "host allocation failed");
  p->masked = true;
  p->prec = precision;
  p->m = m;
  p->n = n;
  p->B = batch;
  p->keep = keep_layers != 0;
  p->inputs.assign(inputs, inputs + (size_t)batch * m);
  p->col.assign((size_t)std::max(n, 1) * batch, 0);
  std::vector<double> inv_in_v(batch);
  for (int b = 0; b < batch; ++b) {
    const std::vector<int> in(inputs + (size_t)b * m, inputs + (size_t)(b + 1) * m);
    const std::vector<int> order = slos_path_order(in);
    for (int k = 0; k < n; ++k) p->col[(size_t)k * batch + b] = order[k];
    double f = 1.0;
    for (int i = 0; i < m; ++i)
      for (int v = 2; v <= in[i]; ++v) f *= v;
    inv_in_v[b] = 1.0 / f;
  }
  const std::vector<uint64_t> inv_in = slos_factor_words(inv_in_v, precision);
  p->sizes.assign(n + 1, 0);
  p->sizes[0] = 1;
  p->mocc_d.assign(n + 1, nullptr);
  p->mpar_d.assign(n + 1, nullptr);
  p->mchild_d.assign(n + 1, nullptr);

  int rc = PCVL_OK;
  const size_t B = (size_t)batch;
  // Cn(M, x) by Pascal's rule, saturating (only ranks of at most C(63, 32) are used)
  const int cs = n + 2;
  std::vector<uint64_t> cn((size_t)(m + 1) * cs, 0);
  for (int M = 0; M <= m; ++M)
    for (int x = 0; x < cs; ++x) {
      uint64_t v;
      if (x == 0)
        v = 1;
      else if (M == 0)
        v = 0;
      else {
        const uint64_t a = cn[(size_t)(M - 1) * cs + x], c = cn[(size_t)M * cs + x - 1];
        v = a > ~0ull - c ? ~0ull : a + c;
      }
      cn[(size_t)M * cs + x] = v;
    }
  TmpBuf cn_d, dg_d, err_d, prev_d, bsum_d, boff_d;
  MaskSpace sp{};
  uint64_t nprev = 1;
  std::vector<uint32_t> bsum;
  std::vector<uint64_t> boff;
  int err_h = 0;
  if ((rc = tmp_alloc(cn_d, cn.size() * 8)) != PCVL_OK) goto fail;
  if ((rc = slos_upload(cn_d.p, cn.data(), cn.size() * 8)) != PCVL_OK) goto fail;
  if ((rc = tmp_alloc(dg_d, (size_t)n_masks * m)) != PCVL_OK) goto fail;
  if ((rc = slos_upload(dg_d.p, digits, (size_t)n_masks * m)) != PCVL_OK) goto fail;
  if ((rc = tmp_alloc(err_d, sizeof(int))) != PCVL_OK) goto fail;
  if (cudaMemset(err_d.p, 0, sizeof(int)) != cudaSuccess) goto cuda_fail;
  if ((rc = tmp_alloc(prev_d, 8)) != PCVL_OK) goto fail;
  if (cudaMemset(prev_d.p, 0, 8) != cudaSuccess) goto cuda_fail;  // layer 0: the vacuum, rank 0
  sp.m = m;
  sp.N = mask_n;
  sp.nmask = n_masks;
  sp.at_least = m >= 32 ? at_least : (at_least & ((1u << m) - 1u));
  sp.cs = cs;
  sp.digits = (const int8_t*)dg_d.p;
  sp.cn = (const uint64_t*)cn_d.p;

  for (int k = 1; k <= n; ++k) {
    if (nprev == 0) break;  // an empty layer empties every later one
    const uint64_t nb = (nprev + kGenThreads - 1) / kGenThreads;
    cudaFree(bsum_d.take());
    cudaFree(boff_d.take());
    if ((rc = tmp_alloc(bsum_d, nb * 4)) != PCVL_OK) goto fail;
    mask_gen<<<(unsigned)nb, kGenThreads>>>(sp, k, (const uint64_t*)prev_d.p, nprev, nullptr,
                                            (uint32_t*)bsum_d.p, nullptr);
    if (cudaGetLastError() != cudaSuccess) goto cuda_fail;
    bsum.resize(nb);
    boff.resize(nb);
    if (cudaMemcpy(bsum.data(), bsum_d.p, nb * 4, cudaMemcpyDeviceToHost) != cudaSuccess) goto cuda_fail;
    uint64_t total = 0;
    for (uint64_t b = 0; b < nb; ++b) {
      boff[b] = total;
      total += bsum[b];
    }
    if (total >= 0xffffffffull) {
      set_error("masked SLOS layer %d keeps %llu states: more than 2^32 - 1 states per layer is not supported", k,
                (unsigned long long)total);
      rc = PCVL_ERR_ARG;
      goto fail;
    }
    p->sizes[k] = total;
    TmpBuf cur;
    if ((rc = tmp_alloc(cur, std::max<uint64_t>(total, 1) * 8)) != PCVL_OK) goto fail;
    if (total > 0) {
      if ((rc = tmp_alloc(boff_d, nb * 8)) != PCVL_OK) goto fail;
      if ((rc = slos_upload(boff_d.p, boff.data(), nb * 8)) != PCVL_OK) goto fail;
      mask_gen<<<(unsigned)nb, kGenThreads>>>(sp, k, (const uint64_t*)prev_d.p, nprev,
                                              (const uint64_t*)boff_d.p, nullptr, (uint64_t*)cur.p);
      if (cudaGetLastError() != cudaSuccess) goto cuda_fail;
    }
    const uint64_t width = (uint64_t)std::min(k, m);
    if ((rc = slos_alloc((void**)&p->mocc_d[k], total * 4, p->bytes)) != PCVL_OK) goto fail;
    if ((rc = slos_alloc((void**)&p->mpar_d[k], width * total * 4, p->bytes)) != PCVL_OK) goto fail;
    if (k == n && (rc = slos_alloc((void**)&p->mfact_d, total * 8, p->bytes)) != PCVL_OK) goto fail;
    if (total > 0) {
      const int run_len = (int)std::max<uint64_t>(
          1, std::min<uint64_t>(kParentRun, total / ((uint64_t)num_sms() * 4096)));
      mask_parents<<<grid_for((total + run_len - 1) / run_len, 8), 256>>>(
          sp, k, (const uint64_t*)cur.p, total, (const uint64_t*)prev_d.p, nprev, p->mocc_d[k], p->mpar_d[k],
          k == n ? p->mfact_d : nullptr, precision == kPrecFP64, (int*)err_d.p, run_len);
      if (cudaGetLastError() != cudaSuccess) goto cuda_fail;
    }
    if (p->keep) {
      if ((rc = slos_alloc((void**)&p->mchild_d[k], (uint64_t)m * nprev * 4, p->bytes)) != PCVL_OK) goto fail;
      if (cudaMemset(p->mchild_d[k], 0xff, (uint64_t)m * nprev * 4) != cudaSuccess) goto cuda_fail;
      if (total > 0) {
        mask_children<<<grid_for(total, 8), 256>>>(p->mocc_d[k], p->mpar_d[k], total, nprev, p->mchild_d[k]);
        if (cudaGetLastError() != cudaSuccess) goto cuda_fail;
      }
    }
    cudaFree(prev_d.take());
    prev_d.p = cur.take();
    nprev = total;
  }
  if (n == 0) {
    // one candidate output, the vacuum: accepted when some mask's digits sum to at most mask_n
    bool vac = false;
    for (int q = 0; q < n_masks && !vac; ++q) {
      int miss = 0;
      for (int i = 0; i < m; ++i) miss += std::max<int>(digits[(size_t)q * m + i], 0);
      vac = miss <= mask_n;
    }
    if (!vac) p->sizes[0] = 0;
    if ((rc = slos_alloc((void**)&p->mfact_d, 8, p->bytes)) != PCVL_OK) goto fail;
    const std::vector<uint64_t> one = slos_factor_words({1.0}, precision);
    if ((rc = slos_upload(p->mfact_d, one.data(), 8)) != PCVL_OK) goto fail;
  }
  if (cudaMemcpy(&err_h, err_d.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) goto cuda_fail;
  if (err_h != 0) {
    set_error("masked SLOS plan: a kept state's parent is missing from the previous layer");
    rc = PCVL_ERR_CUDA;
    goto fail;
  }
  if (p->sizes[n] == 0 || nprev == 0) {
    // nothing accepted: keep an empty rank list
    cudaFree(prev_d.take());
    for (int k = 0; k <= n; ++k)
      if (k > 0 && p->sizes[k - 1] == 0) p->sizes[k] = 0;
  }
  p->mrank_d = (uint64_t*)prev_d.take();
  if (!p->mrank_d && (rc = slos_alloc((void**)&p->mrank_d, 8, p->bytes)) != PCVL_OK) goto fail;
  p->bytes += (int64_t)(p->sizes[n] * 8);

  {
    // coefficient layers, the unitary's columns and (keep) the adjoint buffers
    size_t need = 0, mx = 1;
    for (int k = 0; k <= n; ++k) mx = std::max<size_t>(mx, p->sizes[k]);
    if (p->keep) {
      for (int k = 0; k <= n; ++k) need += p->sizes[k] * B * sizeof(cdd);
      need += 2 * mx * B * sizeof(cdd);
    } else {
      need += 2 * mx * B * sizeof(cdd);
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && need > free_b) {
      set_error("masked SLOS plan needs %zu more bytes of device memory, %zu are free", need, free_b);
      rc = PCVL_ERR_MEMORY;
      goto fail;
    }
    if ((rc = slos_alloc((void**)&p->col_d, p->col.size() * 4, p->bytes)) != PCVL_OK) goto fail;
    if ((rc = slos_upload(p->col_d, p->col.data(), p->col.size() * 4)) != PCVL_OK) goto fail;
    if ((rc = slos_alloc((void**)&p->inv_in_d, B * 8, p->bytes)) != PCVL_OK) goto fail;
    if ((rc = slos_upload(p->inv_in_d, inv_in.data(), B * 8)) != PCVL_OK) goto fail;
    if ((rc = slos_alloc((void**)&p->ucols_d, (size_t)std::max(n, 1) * m * B * sizeof(cdd), p->bytes)) != PCVL_OK)
      goto fail;
    if (p->keep) {
      p->layers.assign(n + 1, nullptr);
      for (int k = 0; k <= n; ++k)  // layer 0 always holds the vacuum of every entry
        if ((rc = slos_alloc((void**)&p->layers[k], std::max<size_t>(p->sizes[k], 1) * B * sizeof(cdd), p->bytes)) !=
            PCVL_OK)
          goto fail;
      for (int i = 0; i < 2; ++i)
        if ((rc = slos_alloc((void**)&p->adj_d[i], mx * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
      p->gpart_blocks = num_sms() * 16;
      if ((rc = slos_alloc((void**)&p->gpart_d, (size_t)p->gpart_blocks * m * B * sizeof(cdd), p->bytes)) !=
          PCVL_OK)
        goto fail;
    } else {
      p->layers.assign(2, nullptr);
      size_t s0 = 1, s1 = 1;
      for (int k = 0; k <= n; ++k) (k % 2 ? s1 : s0) = std::max<size_t>(k % 2 ? s1 : s0, p->sizes[k]);
      if ((rc = slos_alloc((void**)&p->layers[0], s0 * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
      if ((rc = slos_alloc((void**)&p->layers[1], s1 * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
    }
  }
  *plan = p;
  return PCVL_OK;
cuda_fail:
  set_error("masked SLOS plan: CUDA error while building the kept-state tables: %s",
            cudaGetErrorString(cudaGetLastError()));
  rc = PCVL_ERR_CUDA;
fail:
  slos_free_plan(p);
  return rc;
}

// Layers 1..n of a masked plan (the unitary's columns and the vacuum are in place).
int slos_masked_forward(pcvl_slos_plan* p, cudaStream_t s) {
  const int m = p->m, B = p->B;
  for (int k = 1; k <= p->n; ++k) {
    const uint64_t L = p->sizes[k];
    if (L == 0) break;
    const cdd* in = p->keep ? p->layers[k - 1] : p->layers[(k - 1) % 2];
    cdd* out = p->keep ? p->layers[k] : p->layers[k % 2];
    const cdd* ucol = p->ucols_d + (size_t)(k - 1) * m * B;
    const bool f64 = p->prec == kPrecFP64;
    if (B == 1) {
      if (f64)
        slos_mfwd<false, Arith64><<<grid_for(L, 8), 256, 0, s>>>((const double2*)in, (double2*)out, p->mocc_d[k],
                                                                 p->mpar_d[k], L, (const double2*)ucol, m, B);
      else
        slos_mfwd<false, ArithFF><<<grid_for(L, 8), 256, 0, s>>>(in, out, p->mocc_d[k], p->mpar_d[k], L, ucol, m,
                                                                 B);
    } else {
      const dim3 grid((unsigned)std::max<uint64_t>(1, std::min<uint64_t>((L + 7) / 8, (uint64_t)num_sms() * 16)),
                      (unsigned)((B + 31) / 32));
      if (f64)
        slos_mfwd<true, Arith64><<<grid, 256, 0, s>>>((const double2*)in, (double2*)out, p->mocc_d[k],
                                                      p->mpar_d[k], L, (const double2*)ucol, m, B);
      else
        slos_mfwd<true, ArithFF><<<grid, 256, 0, s>>>(in, out, p->mocc_d[k], p->mpar_d[k], L, ucol, m, B);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("masked SLOS layer %d launch failed: %s", k, cudaGetErrorString(e));
      return PCVL_ERR_CUDA;
    }
  }
  return PCVL_OK;
}

int slos_masked_finalize(pcvl_slos_plan* p, int mode, const double* w, double* out_real, double2* out_c,
                         void* seed, cudaStream_t s) {
  const uint64_t L = p->sizes[p->n];
  if (L == 0) return PCVL_OK;
  if (p->prec == kPrecFP64)
    slos_mfin<Arith64><<<grid_for(L * p->B, 8), 256, 0, s>>>(
        (const double2*)p->final_layer(), (const double*)p->mfact_d, (const double*)p->inv_in_d, L, p->B, mode, w,
        out_real, out_c, (double2*)seed);
  else
    slos_mfin<ArithFF><<<grid_for(L * p->B, 8), 256, 0, s>>>(p->final_layer(), p->mfact_d, p->inv_in_d, L, p->B,
                                                             mode, w, out_real, out_c, (cdd*)seed);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

int slos_masked_backward(pcvl_slos_plan* p, const double* weights_d, double* grad_u_d, cudaStream_t s) {
  const int m = p->m, B = p->B, n = p->n;
  PCVL_CUDA(cudaMemsetAsync(grad_u_d, 0, (size_t)B * m * m * 2 * sizeof(double), s));
  if (n == 0 || p->sizes[n] == 0) return PCVL_OK;
  PCVL_TRY(slos_masked_finalize(p, 2, weights_d, nullptr, nullptr, p->adj_d[n % 2], s));
  const bool batched = B > 1;
  for (int k = n; k >= 1; --k) {
    const uint64_t Lp = p->sizes[k - 1];
    const uint64_t units = batched ? (Lp + 7) / 8 : (Lp + 255) / 256;
    const int gx = (int)std::max<uint64_t>(1, std::min<uint64_t>(units, (uint64_t)p->gpart_blocks));
    const dim3 grid((unsigned)gx, batched ? (unsigned)((B + 31) / 32) : 1u);
    const cdd* ain = p->adj_d[k % 2];
    cdd* aout = p->adj_d[(k - 1) % 2];
    const cdd* ucol = p->ucols_d + (size_t)(k - 1) * m * B;
    if (p->prec == kPrecFP64)
      launch_mbwd_m<Arith64>(batched, grid, ain, aout, p->layers[k - 1], p->mchild_d[k], Lp, ucol, m, B,
                             p->gpart_d, s);
    else
      launch_mbwd_m<ArithFF>(batched, grid, ain, aout, p->layers[k - 1], p->mchild_d[k], Lp, ucol, m, B,
                             p->gpart_d, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("masked SLOS adjoint layer %d launch failed: %s", k, cudaGetErrorString(e));
      return PCVL_ERR_CUDA;
    }
    if (p->prec == kPrecFP64)
      slos_mgrad_reduce<Arith64><<<(m * B + 255) / 256, 256, 0, s>>>(
          (const double2*)p->gpart_d, gx, m, B, p->col_d + (size_t)(k - 1) * B, (double2*)grad_u_d);
    else
      slos_mgrad_reduce<ArithFF><<<(m * B + 255) / 256, 256, 0, s>>>(
          p->gpart_d, gx, m, B, p->col_d + (size_t)(k - 1) * B, (double2*)grad_u_d);
    PCVL_CUDA(cudaGetLastError());
  }
  return PCVL_OK;
}

}  // namespace pcvl

using namespace pcvl;

extern "C" int pcvl_slos_plan_create_masked(pcvl_slos_plan** plan, int32_t m, const int32_t* input_states_h,
                                            int32_t batch, int32_t keep_layers, int32_t n_masks,
                                            const int8_t* digits_h, uint32_t at_least_modes, int32_t mask_n,
                                            int32_t precision) {
  return slos_masked_create(plan, m, input_states_h, batch, keep_layers, n_masks, digits_h, at_least_modes, mask_n,
                            precision);
}

extern "C" int pcvl_slos_output_ranks(const pcvl_slos_plan* plan, uint64_t* ranks_h) {
  PCVL_CHECK(plan && ranks_h, "null pointer argument");
  const uint64_t L = plan->sizes[plan->n];
  if (!plan->masked) {
    for (uint64_t i = 0; i < L; ++i) ranks_h[i] = i;
    return PCVL_OK;
  }
  if (L > 0) PCVL_CUDA(cudaMemcpy(ranks_h, plan->mrank_d, L * 8, cudaMemcpyDeviceToHost));
  return PCVL_OK;
}
