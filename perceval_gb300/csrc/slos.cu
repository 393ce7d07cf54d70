// SLOS: layer-by-layer Fock-state amplitude propagation, its adjoint, and the
// normalisation of the last layer into probabilities / amplitudes.
//
// Semantics follow perceval/backends/_slos.py:37-223.  Photons are added one input
// mode at a time in the order of _Path._decompose (:61-86: repeatedly the mode with
// the most remaining photons, first index on ties).  With u_j = U[j, mk] for the
// layer's input mode mk, the k-photon coefficients are
//     c_k[s] = sum_{j : s_j >= 1} u_j c_{k-1}[s - e_j]
// (the gather form of FSMap.compute_slos_layer, whose scatter form the symbolic
// twin at :93-97 spells out).  Amplitude = c_n[s] sqrt(prod s! / prod t!) (:192),
// probability = |c_n[s]|^2 prod s! / prod t! (:198-199, all_prob_normalize_output).
//
// Indexing.  Layer k is the k-photon space in descending lexicographic order.  With
// Cn(M, x) = C(M + x - 1, x) (states of x photons on M modes) and R_{i+1} the photons
// in modes after i:
//     rank(s)          = sum_{i <= m-2} Cn(m - i, R_{i+1} - 1)
//     rank(s - e_j)    = rank(s) - sum_{i < j} Cn(m - i - 1, R_{i+1}(s) - 1)
//     rank(p + e_j)    = rank(p) + sum_{i < j} Cn(m - i - 1, R_{i+1}(p))
// so every parent (child) index comes from one walk over the modes while the state
// is unranked; no parent tables are stored.
//
// Layout.  Coefficients are float-float complex (16 bytes, FP64-class precision),
// state-major with the circuit index b innermost: element (r, b) at r * B + b.  For
// B >= 2 one warp handles one state and its lanes 32 circuits (blockIdx.y selects
// the 32-circuit chunk), so the index walk is warp-uniform and loads are coalesced
// across circuits; for B == 1 each thread handles one state.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "runtime.cuh"

namespace pcvl {

constexpr int kSlosMaxM = 32;
constexpr int kSlosMaxN = 32;
constexpr uint32_t kNone = 0xffffffffu;

struct SlosLayerArgs {
  int m, k, B;
  uint32_t nstates;        // states of the layer written (children fwd, parents bwd)
  const cdd* in;           // layer read
  cdd* out;                // layer written
  const cdd* ucol;         // column mk of every circuit: [j][b]
  const uint32_t* cn;      // Cn table, (m + 1) x (nmax + 1), row M = Cn(M, .)
  int cn_stride;           // nmax + 1
  const cdd* cpar;         // backward: forward coefficients of the parent layer
  cdd* gpart;              // backward: per-CTA partial dL/du_j, [blockIdx.x][j][b]
};

__device__ __forceinline__ uint32_t cn_at(const uint32_t* cn, int stride, int M, int x) {
  return x < 0 ? 0u : cn[M * stride + x];
}

// Unranks child `c` (k photons) and returns the rank of every parent c - e_j
// (kNone where s_j == 0).
template <int MMAX>
__device__ __forceinline__ void parent_ranks(uint32_t c, int m, int k, const uint32_t* cn, int st,
                                             uint32_t (&pr)[MMAX]) {
  uint32_t rho = c, pfx = 0;
  int R = k;
#pragma unroll
  for (int j = 0; j < MMAX; ++j) {
    if (j < m) {
      int v;
      if (j == m - 1) {
        v = R;
      } else {
        const int M1 = m - j;
        int x = R;
        while (x > 0) {
          const uint32_t t = cn_at(cn, st, M1, x - 1);
          if (rho >= t) {
            rho -= t;
            break;
          }
          --x;
        }
        v = R - x;
      }
      pr[j] = v > 0 ? c - pfx : kNone;
      const int Rn = R - v;
      if (j < m - 1) pfx += cn_at(cn, st, m - j - 1, Rn - 1);
      R = Rn;
    } else {
      pr[j] = kNone;
    }
  }
}

// Unranks parent `p` (k photons) and returns the rank of every child p + e_j.
template <int MMAX>
__device__ __forceinline__ void child_ranks(uint32_t p, int m, int k, const uint32_t* cn, int st,
                                            uint32_t (&ch)[MMAX]) {
  uint32_t rho = p, q = 0;
  int R = k;
#pragma unroll
  for (int j = 0; j < MMAX; ++j) {
    if (j < m) {
      ch[j] = p + q;
      int v;
      if (j == m - 1) {
        v = R;
      } else {
        const int M1 = m - j;
        int x = R;
        while (x > 0) {
          const uint32_t t = cn_at(cn, st, M1, x - 1);
          if (rho >= t) {
            rho -= t;
            break;
          }
          --x;
        }
        v = R - x;
      }
      const int Rn = R - v;
      if (j < m - 1) q += cn_at(cn, st, m - j - 1, Rn);
      R = Rn;
    } else {
      ch[j] = kNone;
    }
  }
}

// Unranks state r and returns prod_j s_j! (as a double).
__device__ __forceinline__ double state_prodfact(uint32_t r, int m, int k, const uint32_t* cn, int st,
                                                 const double* fact) {
  uint32_t rho = r;
  int R = k;
  double pf = 1.0;
  for (int j = 0; j < m && R > 0; ++j) {
    int v;
    if (j == m - 1) {
      v = R;
    } else {
      const int M1 = m - j;
      int x = R;
      while (x > 0) {
        const uint32_t t = cn_at(cn, st, M1, x - 1);
        if (rho >= t) {
          rho -= t;
          break;
        }
        --x;
      }
      v = R - x;
    }
    pf *= fact[v];
    R -= v;
  }
  return pf;
}

// ------------------------------------------------------------------ tiled single-circuit path
// The modes split into a prefix (the first p = m - t) and a tail (the last t <= 8).
// A tile is the set of states sharing one prefix pi; its r = k - |pi| tail photons
// range over the count(t, r) tail states tau, contiguous in rank order:
//     rank(pi, tau) = A(pi, r) + rank_t(tau),  A = sum_{i<p} Cn(m - i, R_{i+1} - 1).
// Tiles themselves are ordered like the states of the (p + 1)-mode space whose last
// mode holds r, so tile index -> pi is one unranking.  Parents of (pi, tau):
//   prefix mode j:  A - Pfx_j + rank_t(tau)          (contiguous over tau)
//   tail mode j:    A - Pfx_p + rank_t(tau - e_j)    (rank_t from a small table)
// with Pfx_j = sum_{i<j} Cn(m - i - 1, R_{i+1} - 1).  Descriptors are computed once per
// tile (one thread each) for a chunk of tiles; the CTA's threads then sweep the
// chunk's children, finding their tile by binary search over the chunk's offsets.
constexpr int kTileChunk = 128;

struct SlosTiledArgs {
  int m, k, p, t;
  uint32_t ntiles;
  const cdd* in;
  cdd* out;
  const cdd* ucol;          // u_j = U[j, mk]
  const uint32_t* cn;
  int cn_stride;
  const uint32_t* tail;     // tail tables: parent ranks (forward) or child ranks (backward)
  uint32_t tail_off[kSlosMaxN + 2];  // entry offset of the block of r tail photons
  uint32_t tstate_off[kSlosMaxN + 2];  // state offset of the block of r tail photons
  uint32_t tsize[kSlosMaxN + 2];     // count(t, r)
};

struct TileDesc {
  uint32_t start, tbase, mask;
  int r;
};

// Descriptor of tile `tile` of layer k; pre[i] receives A - Pfx_i for occupied
// prefix modes (bit i of mask).
template <int MMAX>
__device__ __forceinline__ TileDesc tile_desc(uint32_t tile, int m, int k, int p, const uint32_t* cn, int st,
                                             uint32_t* pre) {
  uint32_t rho = tile, A = 0, Pfx = 0, mask = 0;
  int R = k;
#pragma unroll
  for (int i = 0; i < MMAX; ++i) {
    if (i < p) {
      const int M1 = p + 1 - i;
      int x = R;
      while (x > 0) {
        const uint32_t c = cn_at(cn, st, M1, x - 1);
        if (rho >= c) {
          rho -= c;
          break;
        }
        --x;
      }
      const int v = R - x;
      if (v > 0) {
        mask |= 1u << i;
        pre[i] = Pfx;
      }
      const int Rn = R - v;
      A += cn_at(cn, st, m - i, Rn - 1);
      Pfx += cn_at(cn, st, m - i - 1, Rn - 1);
      R = Rn;
    }
  }
#pragma unroll
  for (int i = 0; i < MMAX; ++i)
    if (i < p && ((mask >> i) & 1u)) pre[i] = A - pre[i];
  return {A, A - Pfx, mask, R};
}

// exclusive scan of kTileChunk sizes held one per thread (threads >= kTileChunk pass 0)
__device__ __forceinline__ void chunk_scan(uint32_t v, uint32_t* off, uint32_t* warp_tot) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (tid < kTileChunk && lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (tid < kTileChunk) {
    uint32_t base = 0;
    for (int q = 0; q < w; ++q) base += warp_tot[q];
    off[tid + 1] = base + x;
    if (tid == 0) off[0] = 0;
  }
  __syncthreads();
}

// mode 0: forward layer (gather from parents); mode 1: adjoint layer (gather from
// children, plus per-CTA partials of dL/du); the parent/child roles swap through the
// tail table and the prefix offsets.
template <int MMAX>
__global__ void __launch_bounds__(256) slos_forward_tiled(SlosTiledArgs a) {
  extern __shared__ uint32_t cn_s[];
  __shared__ uint32_t s_off[kTileChunk + 1], s_start[kTileChunk], s_tbase[kTileChunk], s_mask[kTileChunk];
  __shared__ int s_r[kTileChunk];
  __shared__ uint32_t s_pre[kTileChunk][MMAX];
  __shared__ uint32_t s_wtot[kTileChunk / 32];
  __shared__ cdd u[MMAX];
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn_s[i] = a.cn[i];
  const int m = a.m, p = a.p, t = a.t, tid = threadIdx.x;
  if (tid < MMAX) u[tid] = tid < m ? a.ucol[tid] : cdd_zero();
  __syncthreads();
  const uint32_t nchunks = (a.ntiles + kTileChunk - 1) / kTileChunk;
  for (uint32_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    // largest tiles (small prefixes) come last in rank order: take chunks from the end
    const uint32_t first = (nchunks - 1 - ch) * kTileChunk;
    uint32_t size = 0;
    if (tid < kTileChunk && first + tid < a.ntiles) {
      const TileDesc d = tile_desc<MMAX>(first + tid, m, a.k, p, cn_s, a.cn_stride, s_pre[tid]);
      s_start[tid] = d.start;
      s_tbase[tid] = d.tbase;
      s_mask[tid] = d.mask;
      s_r[tid] = d.r;
      size = a.tsize[d.r];
    }
    chunk_scan(size, s_off, s_wtot);
    const uint32_t total = s_off[kTileChunk];
    for (uint32_t idx = tid; idx < total; idx += blockDim.x) {
      int lo = 0, hi = kTileChunk;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s_off[mid] <= idx) lo = mid; else hi = mid;
      }
      const uint32_t tau = idx - s_off[lo];
      const uint32_t mask = s_mask[lo];
      const int r = s_r[lo];
      const uint32_t tbase = s_tbase[lo];
      const uint32_t* row = a.tail + a.tail_off[r] + (size_t)tau * t;
      cacc acc = cacc_zero();
#pragma unroll
      for (int j = 0; j < MMAX; ++j) {
        if (j < p) {
          if ((mask >> j) & 1u) cacc_fma(acc, ld_cdd(&a.in[s_pre[lo][j] + tau]), u[j]);
        } else if (j < m && r > 0) {
          const uint32_t e = __ldg(&row[j - p]);
          if (e != kNone) cacc_fma(acc, ld_cdd(&a.in[tbase + e]), u[j]);
        }
      }
      a.out[s_start[lo] + tau] = cacc_finish(acc);
    }
    __syncthreads();
  }
}

// double from a float by exponent re-bias (integer pipe); zero and subnormals take the
// conversion instruction
__device__ __forceinline__ double f2d_int(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const uint64_t bits = ((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                        ((uint64_t)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}
__device__ __forceinline__ double dd_to_double_fast(dd a) { return f2d_int(a.hi) + f2d_int(a.lo); }

// Probabilities (mode 0), amplitudes (mode 1) or adjoint seed (mode 2) of the last
// layer over tiles: F = prod(out!) / prod(in!) = fpre (per tile, float-float) x ftail[tau].
template <int MMAX>
__global__ void __launch_bounds__(256) slos_finalize_tiled(SlosTiledArgs a, const dd* __restrict__ ftail,
                                                          dd inv_in, int mode, const double* __restrict__ w,
                                                          double* __restrict__ out_real, double2* __restrict__ out_c,
                                                          cdd* __restrict__ seed) {
  extern __shared__ uint32_t cn_s[];
  __shared__ uint32_t s_off[kTileChunk + 1], s_start[kTileChunk];
  __shared__ int s_r[kTileChunk];
  __shared__ dd s_f[kTileChunk];
  __shared__ uint32_t s_wtot[kTileChunk / 32];
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn_s[i] = a.cn[i];
  __syncthreads();
  const int m = a.m, p = a.p, tid = threadIdx.x;
  const uint32_t nchunks = (a.ntiles + kTileChunk - 1) / kTileChunk;
  for (uint32_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const uint32_t first = (nchunks - 1 - ch) * kTileChunk;
    uint32_t size = 0;
    if (tid < kTileChunk && first + tid < a.ntiles) {
      // prefix occupation: unrank the tile again, multiplying the factorials
      uint32_t rho = first + tid;
      int R = a.k;
      dd f = inv_in;
      uint32_t A = 0;
      for (int i = 0; i < p; ++i) {
        const int M1 = p + 1 - i;
        int x = R;
        while (x > 0) {
          const uint32_t c = cn_at(cn_s, a.cn_stride, M1, x - 1);
          if (rho >= c) {
            rho -= c;
            break;
          }
          --x;
        }
        const int v = R - x;
        for (int q = 2; q <= v; ++q) f = dd_mul_f(f, (float)q);
        const int Rn = R - v;
        A += cn_at(cn_s, a.cn_stride, m - i, Rn - 1);
        R = Rn;
      }
      s_start[tid] = A;
      s_r[tid] = R;
      s_f[tid] = f;
      size = a.tsize[R];
    }
    chunk_scan(size, s_off, s_wtot);
    const uint32_t total = s_off[kTileChunk];
    for (uint32_t idx = tid; idx < total; idx += blockDim.x) {
      int lo = 0, hi = kTileChunk;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s_off[mid] <= idx) lo = mid; else hi = mid;
      }
      const uint32_t tau = idx - s_off[lo];
      const uint32_t r_idx = s_start[lo] + tau;
      const dd F = dd_mul(s_f[lo], ftail[a.tstate_off[s_r[lo]] + tau]);
      const cdd c = ld_cdd(&a.in[r_idx]);
      if (mode == 0) {
        const dd c2 = dd_add(dd_mul(c.re, c.re), dd_mul(c.im, c.im));
        out_real[r_idx] = dd_to_double_fast(dd_mul(c2, F));
      } else if (mode == 1) {
        const double sF = sqrt(dd_to_double_fast(F));
        out_c[r_idx] = make_double2(dd_to_double_fast(c.re) * sF, dd_to_double_fast(c.im) * sF);
      } else {
        const dd f2 = dd_mul(dd_from_double(2.0 * w[r_idx]), F);
        seed[r_idx] = {dd_mul(c.re, f2), dd_mul(c.im, f2)};
      }
    }
    __syncthreads();
  }
}

template <int MMAX, bool BATCHED>
__global__ void __launch_bounds__(256) slos_forward_layer(SlosLayerArgs a) {
  extern __shared__ uint32_t cn_s[];
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn_s[i] = a.cn[i];
  __syncthreads();
  const int m = a.m, B = a.B;
  if (!BATCHED) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < a.nstates; c += gridDim.x * blockDim.x) {
      uint32_t pr[MMAX];
      parent_ranks<MMAX>(c, m, a.k, cn_s, a.cn_stride, pr);
      cacc acc = cacc_zero();
#pragma unroll
      for (int j = 0; j < MMAX; ++j)
        if (pr[j] != kNone) cacc_fma(acc, ld_cdd(&a.in[pr[j]]), ld_cdd(&a.ucol[j]));
      a.out[c] = cacc_finish(acc);
    }
  } else {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.y * 32 + lane;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    cdd u[MMAX];
#pragma unroll
    for (int j = 0; j < MMAX; ++j) u[j] = (j < m && b < B) ? a.ucol[(size_t)j * B + b] : cdd_zero();
    for (uint32_t c = warp; c < a.nstates; c += nwarps) {
      uint32_t pr[MMAX];
      parent_ranks<MMAX>(c, m, a.k, cn_s, a.cn_stride, pr);
      if (b < B) {
        cacc acc = cacc_zero();
#pragma unroll
        for (int j = 0; j < MMAX; ++j)
          if (pr[j] != kNone) cacc_fma(acc, ld_cdd(&a.in[(size_t)pr[j] * B + b]), u[j]);
        a.out[(size_t)c * B + b] = cacc_finish(acc);
      }
    }
  }
}

// One adjoint step: parent adjoint a_{k-1}[p] = sum_j conj(u_j) a_k[p + e_j] and the
// per-CTA partial of dL/du_j = sum_p conj(c_{k-1}[p]) a_k[p + e_j].
template <int MMAX, bool BATCHED>
__global__ void __launch_bounds__(256) slos_backward_layer(SlosLayerArgs a) {
  extern __shared__ uint32_t cn_s[];
  __shared__ cdd red[8][32];
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn_s[i] = a.cn[i];
  __syncthreads();
  const int m = a.m, B = a.B;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  cacc g[MMAX];
#pragma unroll
  for (int j = 0; j < MMAX; ++j) g[j] = cacc_zero();

  if (!BATCHED) {
    cdd uc[MMAX];
#pragma unroll
    for (int j = 0; j < MMAX; ++j) uc[j] = j < m ? cdd_conj(a.ucol[j]) : cdd_zero();
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < a.nstates; p += gridDim.x * blockDim.x) {
      uint32_t ch[MMAX];
      child_ranks<MMAX>(p, m, a.k, cn_s, a.cn_stride, ch);
      const cdd cp = cdd_conj(a.cpar[p]);
      cacc acc = cacc_zero();
#pragma unroll
      for (int j = 0; j < MMAX; ++j) {
        if (j < m) {
          const cdd x = ld_cdd(&a.in[ch[j]]);
          cacc_fma(acc, x, uc[j]);
          cacc_fma(g[j], x, cp);
        }
      }
      a.out[p] = cacc_finish(acc);
    }
    // block reduction of g[j] over all threads; thread 0 of the block writes
#pragma unroll
    for (int j = 0; j < MMAX; ++j) {
      if (j >= m) break;
      cdd v = cacc_finish(g[j]);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) {
        cdd o;
        o.re.hi = __shfl_down_sync(0xffffffffu, v.re.hi, d);
        o.re.lo = __shfl_down_sync(0xffffffffu, v.re.lo, d);
        o.im.hi = __shfl_down_sync(0xffffffffu, v.im.hi, d);
        o.im.lo = __shfl_down_sync(0xffffffffu, v.im.lo, d);
        v = cdd_add(v, o);
      }
      if (lane == 0) red[wid][0] = v;
      __syncthreads();
      if (threadIdx.x == 0) {
        cdd s = red[0][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s = cdd_add(s, red[w][0]);
        a.gpart[(size_t)blockIdx.x * m + j] = s;
      }
      __syncthreads();
    }
  } else {
    const int b = blockIdx.y * 32 + lane;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    cdd uc[MMAX];
#pragma unroll
    for (int j = 0; j < MMAX; ++j) uc[j] = (j < m && b < B) ? cdd_conj(a.ucol[(size_t)j * B + b]) : cdd_zero();
    for (uint32_t p = warp; p < a.nstates; p += nwarps) {
      uint32_t ch[MMAX];
      child_ranks<MMAX>(p, m, a.k, cn_s, a.cn_stride, ch);
      if (b < B) {
        const cdd cp = cdd_conj(a.cpar[(size_t)p * B + b]);
        cacc acc = cacc_zero();
#pragma unroll
        for (int j = 0; j < MMAX; ++j) {
          if (j < m) {
            const cdd x = ld_cdd(&a.in[(size_t)ch[j] * B + b]);
            cacc_fma(acc, x, uc[j]);
            cacc_fma(g[j], x, cp);
          }
        }
        a.out[(size_t)p * B + b] = cacc_finish(acc);
      }
    }
    // reduce g[j] over the warps of the block, per lane (= circuit)
#pragma unroll
    for (int j = 0; j < MMAX; ++j) {
      if (j >= m) break;
      red[wid][lane] = cacc_finish(g[j]);
      __syncthreads();
      if (wid == 0) {
        cdd s = red[0][lane];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s = cdd_add(s, red[w][lane]);
        if (b < B) a.gpart[((size_t)blockIdx.x * m + j) * B + b] = s;
      }
      __syncthreads();
    }
  }
}

// grad[b][j][mk] += sum over CTAs of gpart[cta][j][b]
__global__ void slos_grad_reduce(const cdd* __restrict__ gpart, int nblk, int m, int B, int mk,
                                 double2* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // i = j * B + b
  if (i >= m * B) return;
  const int j = i / B, b = i - j * B;
  cdd s = cdd_zero();
  for (int q = 0; q < nblk; ++q) s = cdd_add(s, gpart[(size_t)q * m * B + i]);
  double2* g = &grad[((size_t)b * m + j) * m + mk];
  g->x += dd_to_double(s.re);
  g->y += dd_to_double(s.im);
}

// ucol[mk][j][b] = U_b[j][mk] as float-float, for every column mk
__global__ void slos_convert_u(const double2* __restrict__ u, int m, int B, cdd* __restrict__ ucols) {
  const size_t tot = (size_t)B * m * m;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t b = i / ((size_t)m * m);
    const int rem = (int)(i - b * m * m);
    const int j = rem / m, col = rem - j * m;
    const double2 v = u[i];
    ucols[((size_t)col * m + j) * B + b] = cdd_from(v.x, v.y);
  }
}

__global__ void slos_fill_vacuum(cdd* layer0, int B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) layer0[b] = cdd_one();
}

// mode 0: probabilities (double), 1: amplitudes (complex128), 2: adjoint seed
// a_n = 2 w F c (needs w), where F = prod(out!) / prod(in!).
__global__ void slos_finalize(const cdd* __restrict__ cfin, uint32_t nstates, int m, int n, int B,
                              const uint32_t* __restrict__ cn, int cn_stride, double inv_prodfact_in,
                              int mode, const double* __restrict__ w, double* __restrict__ out_real,
                              double2* __restrict__ out_cplx, cdd* __restrict__ seed) {
  __shared__ double fact[kSlosMaxN + 1];
  extern __shared__ uint32_t cn_s[];
  if (threadIdx.x <= kSlosMaxN) {
    double f = 1.0;
    for (int i = 2; i <= (int)threadIdx.x; ++i) f *= i;
    fact[threadIdx.x] = f;
  }
  const int ncn = (m + 1) * cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn_s[i] = cn[i];
  __syncthreads();
  const size_t tot = (size_t)nstates * B;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(i / B);
    const double F = state_prodfact(r, m, n, cn_s, cn_stride, fact) * inv_prodfact_in;
    const cdd c = cfin[i];
    if (mode == 0) {
      const dd c2 = dd_add(dd_mul(c.re, c.re), dd_mul(c.im, c.im));
      out_real[i] = dd_to_double(c2) * F;
    } else if (mode == 1) {
      const double s = sqrt(F);
      out_cplx[i] = make_double2(dd_to_double(c.re) * s, dd_to_double(c.im) * s);
    } else {
      const double f = 2.0 * w[i] * F;
      const dd fd = dd_from_double(f);
      seed[i] = {dd_mul(c.re, fd), dd_mul(c.im, fd)};
    }
  }
}

template <int MMAX>
static int launch_layer(bool backward, const SlosLayerArgs& a, int grid, cudaStream_t s) {
  const size_t smem = (size_t)(a.m + 1) * a.cn_stride * sizeof(uint32_t);
  const bool batched = a.B > 1;
  dim3 g(grid, batched ? (a.B + 31) / 32 : 1);
  if (!backward) {
    if (batched)
      slos_forward_layer<MMAX, true><<<g, 256, smem, s>>>(a);
    else
      slos_forward_layer<MMAX, false><<<g, 256, smem, s>>>(a);
  } else {
    if (batched)
      slos_backward_layer<MMAX, true><<<g, 256, smem, s>>>(a);
    else
      slos_backward_layer<MMAX, false><<<g, 256, smem, s>>>(a);
  }
  return (int)cudaGetLastError();
}

static int dispatch_layer(bool backward, const SlosLayerArgs& a, int grid, cudaStream_t s) {
  if (a.m <= 8) return launch_layer<8>(backward, a, grid, s);
  if (a.m <= 16) return launch_layer<16>(backward, a, grid, s);
  if (a.m <= 24) return launch_layer<24>(backward, a, grid, s);
  return launch_layer<32>(backward, a, grid, s);
}

}  // namespace pcvl

using namespace pcvl;

struct pcvl_slos_plan {
  int m = 0, n = 0, B = 0;
  bool keep = false;
  std::vector<int> input;
  std::vector<int> order;         // input mode of photon k (k = 1..n) -> order[k-1]
  std::vector<uint64_t> sizes;    // layer sizes, k = 0..n
  double prodfact_in = 1.0;
  int cn_stride = 0;
  uint32_t* cn_d = nullptr;
  cdd* ucols_d = nullptr;         // [col][j][b]
  std::vector<cdd*> layers;       // keep: every layer; else layers[k % 2] ping-pong
  cdd* adj_d[2] = {nullptr, nullptr};
  cdd* gpart_d = nullptr;
  int gpart_blocks = 0;
  int64_t bytes = 0;
  bool forwarded = false;
  // tiled single-circuit path (batch == 1)
  int tail_t = 0, tail_p = 0;
  uint32_t* tail_parent_d = nullptr;   // rank_t(tau - e_j) per tail state and tail mode
  dd* ftail_d = nullptr;               // prod tau_j! per tail state
  std::vector<uint32_t> tail_off, tstate_off, tsize;
  cdd* final_layer() const { return keep ? layers[n] : layers[n % 2]; }
};

namespace {

void free_plan(pcvl_slos_plan* p) {
  if (!p) return;
  cudaFree(p->cn_d);
  cudaFree(p->ucols_d);
  for (cdd* l : p->layers) cudaFree(l);
  cudaFree(p->adj_d[0]);
  cudaFree(p->adj_d[1]);
  cudaFree(p->gpart_d);
  cudaFree(p->tail_parent_d);
  cudaFree(p->ftail_d);
  delete p;
}

// Tail tables for t tail modes and up to n tail photons (descending-lex order within
// each photon number): parent ranks rank_t(tau - e_j) (kNone where tau_j = 0) and the
// factorial products prod_j tau_j!.
void tail_tables(int t, int n, std::vector<uint32_t>& parent, std::vector<dd>& ftail, std::vector<uint32_t>& tail_off,
                 std::vector<uint32_t>& tstate_off, std::vector<uint32_t>& tsize) {
  tail_off.assign(n + 2, 0);
  tstate_off.assign(n + 2, 0);
  tsize.assign(n + 2, 0);
  parent.clear();
  ftail.clear();
  auto rank = [t](const std::vector<int>& s) {
    int rest = 0;
    for (int v : s) rest += v;
    uint64_t r = 0;
    for (int i = 0; i < t; ++i) {
      rest -= s[i];
      if (rest > 0) r += fock_count(t - i, rest - 1);
    }
    return (uint32_t)r;
  };
  for (int r = 0; r <= n; ++r) {
    tail_off[r] = (uint32_t)parent.size();
    tstate_off[r] = (uint32_t)ftail.size();
    tsize[r] = (uint32_t)fock_count(t, r);
    std::vector<int> s(t, 0);
    s[0] = r;
    for (uint32_t q = 0; q < tsize[r]; ++q) {
      double f = 1.0;
      for (int j = 0; j < t; ++j) {
        for (int v = 2; v <= s[j]; ++v) f *= v;
        if (s[j] == 0) {
          parent.push_back(kNone);
        } else {
          s[j] -= 1;
          parent.push_back(rank(s));
          s[j] += 1;
        }
      }
      ftail.push_back(dd_from_double(f));
      // next state in descending-lex order
      int tail = 0;
      for (int i = t - 2; i >= 0; --i) {
        tail += s[i + 1];
        if (s[i] > 0) {
          s[i] -= 1;
          s[i + 1] = tail + 1;
          for (int j = i + 2; j < t; ++j) s[j] = 0;
          break;
        }
      }
    }
  }
  tail_off[n + 1] = (uint32_t)parent.size();
  tstate_off[n + 1] = (uint32_t)ftail.size();
}

// Photon-addition order of perceval/backends/_slos.py:61-86 for one input state:
// repeatedly take the mode with the largest remaining count (first index on ties).
std::vector<int> path_order(const std::vector<int>& input) {
  std::vector<int> cnt(input), order;
  while (true) {
    int best = -1, bv = 0;
    for (size_t i = 0; i < cnt.size(); ++i)
      if (cnt[i] > bv) {
        bv = cnt[i];
        best = (int)i;
      }
    if (best < 0) break;
    order.push_back(best);
    --cnt[best];
  }
  return order;
}

int alloc(void** p, size_t bytes, int64_t& total) {
  cudaError_t e = cudaMalloc(p, bytes < 256 ? 256 : bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    pcvl::set_error("SLOS plan: device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return PCVL_ERR_MEMORY;
  }
  total += (int64_t)bytes;
  return PCVL_OK;
}

int grid_for(uint64_t work_units, int per_block) {
  const int sms = pcvl::num_sms();
  uint64_t g = (work_units + per_block - 1) / per_block;
  g = std::min<uint64_t>(g, (uint64_t)sms * 16);
  return (int)std::max<uint64_t>(g, 1);
}

}  // namespace

extern "C" int pcvl_slos_plan_create(pcvl_slos_plan** plan, int32_t m, const int32_t* input_state_h,
                                     int32_t batch, int32_t keep_layers) {
  PCVL_CHECK(plan && input_state_h, "null pointer argument");
  *plan = nullptr;
  PCVL_CHECK(m >= 1 && m <= kSlosMaxM, "m=%d outside [1, %d]", m, kSlosMaxM);
  PCVL_CHECK(batch >= 1, "batch must be >= 1");
  int n = 0;
  for (int i = 0; i < m; ++i) {
    PCVL_CHECK(input_state_h[i] >= 0, "negative photon count in input state");
    n += input_state_h[i];
  }
  PCVL_CHECK(n <= kSlosMaxN, "n=%d photons exceeds %d", n, kSlosMaxN);

  auto* p = new (std::nothrow) pcvl_slos_plan();
  PCVL_CHECK(p, "host allocation failed");
  p->m = m;
  p->n = n;
  p->B = batch;
  p->keep = keep_layers != 0;
  p->input.assign(input_state_h, input_state_h + m);
  p->order = path_order(p->input);
  for (int i = 0; i < m; ++i)
    for (int v = 2; v <= p->input[i]; ++v) p->prodfact_in *= v;
  p->sizes.resize(n + 1);
  for (int k = 0; k <= n; ++k) {
    p->sizes[k] = fock_count(m, k);
    if (p->sizes[k] >= 0xffffffffull) {
      delete p;
      set_error("SLOS layer %d holds %llu states: more than 2^32 - 1 states per layer is not supported",
                k, (unsigned long long)fock_count(m, k));
      return PCVL_ERR_ARG;
    }
  }
  // predicted footprint, refused before any allocation
  const size_t B = (size_t)batch;
  size_t need = 0;
  if (p->keep) {
    for (int k = 0; k <= n; ++k) need += p->sizes[k] * B * sizeof(cdd);
    size_t mx = 0;
    for (int k = 0; k <= n; ++k) mx = std::max<size_t>(mx, p->sizes[k]);
    need += 2 * mx * B * sizeof(cdd);
  } else {
    need += (p->sizes[n] + (n > 0 ? p->sizes[n - 1] : 0)) * B * sizeof(cdd);
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && need > free_b) {
    delete p;
    set_error("SLOS plan needs %zu bytes of device memory, %zu are free", need, free_b);
    return PCVL_ERR_MEMORY;
  }

  int rc = PCVL_OK;
  p->cn_stride = n + 1;
  std::vector<uint32_t> cn((size_t)(m + 1) * p->cn_stride);
  for (int M = 0; M <= m; ++M)
    for (int x = 0; x <= n; ++x) cn[(size_t)M * p->cn_stride + x] = (uint32_t)fock_count(M, x);
  if ((rc = alloc((void**)&p->cn_d, cn.size() * 4, p->bytes)) != PCVL_OK) goto fail;
  if (cudaMemcpy(p->cn_d, cn.data(), cn.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("SLOS plan: table upload failed");
    rc = PCVL_ERR_CUDA;
    goto fail;
  }
  if ((rc = alloc((void**)&p->ucols_d, (size_t)m * m * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
  if (p->keep) {
    p->layers.assign(n + 1, nullptr);
    for (int k = 0; k <= n; ++k)
      if ((rc = alloc((void**)&p->layers[k], p->sizes[k] * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
    size_t mx = 0;
    for (int k = 0; k <= n; ++k) mx = std::max<size_t>(mx, p->sizes[k]);
    for (int i = 0; i < 2; ++i)
      if ((rc = alloc((void**)&p->adj_d[i], mx * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
    p->gpart_blocks = pcvl::num_sms() * 4;
    if ((rc = alloc((void**)&p->gpart_d, (size_t)p->gpart_blocks * m * B * sizeof(cdd), p->bytes)) != PCVL_OK)
      goto fail;
  } else {
    p->layers.assign(2, nullptr);
    size_t s0 = 0, s1 = 0;
    for (int k = 0; k <= n; ++k) (k % 2 ? s1 : s0) = std::max<size_t>(k % 2 ? s1 : s0, p->sizes[k]);
    if ((rc = alloc((void**)&p->layers[0], s0 * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
    if ((rc = alloc((void**)&p->layers[1], std::max<size_t>(s1, 1) * B * sizeof(cdd), p->bytes)) != PCVL_OK)
      goto fail;
  }
  if (batch == 1) {
    // largest tail (<= 8 modes, < m so the prefix is non-empty unless m == 1) whose
    // tables stay small: count(t + 1, n) tail states over all photon numbers
    int t = std::min(m, 8);
    while (t > 1 && fock_count(t + 1, n) > 1000000ull) --t;
    p->tail_t = t;
    p->tail_p = m - t;
    std::vector<uint32_t> parent;
    std::vector<dd> ftail;
    tail_tables(t, n, parent, ftail, p->tail_off, p->tstate_off, p->tsize);
    if ((rc = alloc((void**)&p->tail_parent_d, parent.size() * 4, p->bytes)) != PCVL_OK) goto fail;
    if ((rc = alloc((void**)&p->ftail_d, ftail.size() * sizeof(dd), p->bytes)) != PCVL_OK) goto fail;
    if (cudaMemcpy(p->tail_parent_d, parent.data(), parent.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(p->ftail_d, ftail.data(), ftail.size() * sizeof(dd), cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("SLOS plan: tail table upload failed");
      rc = PCVL_ERR_CUDA;
      goto fail;
    }
  }
  *plan = p;
  return PCVL_OK;
fail:
  free_plan(p);
  return rc;
}

static SlosTiledArgs tiled_args(const pcvl_slos_plan* p, int k) {
  SlosTiledArgs a{};
  a.m = p->m;
  a.k = k;
  a.p = p->tail_p;
  a.t = p->tail_t;
  a.ntiles = (uint32_t)fock_count(p->tail_p + 1, k);
  a.cn = p->cn_d;
  a.cn_stride = p->cn_stride;
  a.tail = p->tail_parent_d;
  for (int r = 0; r <= p->n + 1 && r < kSlosMaxN + 2; ++r) {
    a.tail_off[r] = p->tail_off[r];
    a.tstate_off[r] = p->tstate_off[r];
    a.tsize[r] = p->tsize[r];
  }
  return a;
}

template <int MMAX>
static int launch_tiled(const SlosTiledArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)(a.m + 1) * a.cn_stride * sizeof(uint32_t);
  const uint32_t chunks = (a.ntiles + kTileChunk - 1) / kTileChunk;
  const int grid = (int)std::max<uint32_t>(1, std::min<uint32_t>(chunks, (uint32_t)num_sms() * 8));
  slos_forward_tiled<MMAX><<<grid, 256, smem, s>>>(a);
  return (int)cudaGetLastError();
}

static int dispatch_tiled(const SlosTiledArgs& a, cudaStream_t s) {
  if (a.m <= 8) return launch_tiled<8>(a, s);
  if (a.m <= 16) return launch_tiled<16>(a, s);
  if (a.m <= 24) return launch_tiled<24>(a, s);
  return launch_tiled<32>(a, s);
}

template <int MMAX>
static int launch_fin_tiled(const SlosTiledArgs& a, const dd* ftail, dd inv_in, int mode, const double* w,
                            double* out_real, double2* out_c, cdd* seed, cudaStream_t s) {
  const size_t smem = (size_t)(a.m + 1) * a.cn_stride * sizeof(uint32_t);
  const uint32_t chunks = (a.ntiles + kTileChunk - 1) / kTileChunk;
  const int grid = (int)std::max<uint32_t>(1, std::min<uint32_t>(chunks, (uint32_t)num_sms() * 8));
  slos_finalize_tiled<MMAX><<<grid, 256, smem, s>>>(a, ftail, inv_in, mode, w, out_real, out_c, seed);
  return (int)cudaGetLastError();
}

extern "C" int pcvl_slos_plan_destroy(pcvl_slos_plan* plan) {
  free_plan(plan);
  return PCVL_OK;
}

extern "C" int pcvl_slos_output_count(const pcvl_slos_plan* plan, int64_t* count) {
  PCVL_CHECK(plan && count, "null pointer argument");
  *count = (int64_t)plan->sizes[plan->n];
  return PCVL_OK;
}

extern "C" int pcvl_slos_plan_bytes(const pcvl_slos_plan* plan, int64_t* bytes) {
  PCVL_CHECK(plan && bytes, "null pointer argument");
  *bytes = plan->bytes;
  return PCVL_OK;
}

extern "C" int pcvl_slos_forward(pcvl_slos_plan* p, const double* u_d, void* stream_) {
  PCVL_CHECK(p && u_d, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream_;
  const int m = p->m, B = p->B;
  slos_convert_u<<<grid_for((uint64_t)B * m * m, 256), 256, 0, s>>>((const double2*)u_d, m, B, p->ucols_d);
  PCVL_CUDA(cudaGetLastError());
  cdd* l0 = p->layers[0];
  slos_fill_vacuum<<<(B + 255) / 256, 256, 0, s>>>(l0, B);
  PCVL_CUDA(cudaGetLastError());
  for (int k = 1; k <= p->n; ++k) {
    SlosLayerArgs a{};
    a.m = m;
    a.k = k;
    a.B = B;
    a.nstates = (uint32_t)p->sizes[k];
    a.in = p->keep ? p->layers[k - 1] : p->layers[(k - 1) % 2];
    a.out = p->keep ? p->layers[k] : p->layers[k % 2];
    a.ucol = p->ucols_d + (size_t)p->order[k - 1] * m * B;
    a.cn = p->cn_d;
    a.cn_stride = p->cn_stride;
    int rc;
    if (B == 1) {
      SlosTiledArgs ta = tiled_args(p, k);
      ta.in = a.in;
      ta.out = a.out;
      ta.ucol = a.ucol;
      rc = dispatch_tiled(ta, s);
    } else {
      rc = dispatch_layer(false, a, grid_for(a.nstates, 8), s);
    }
    if (rc != 0) {
      set_error("SLOS layer %d launch failed: %s", k, cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
  }
  p->forwarded = true;
  return PCVL_OK;
}

static int finalize(pcvl_slos_plan* p, int mode, const double* w, double* out_real, double2* out_c, cdd* seed,
                    cudaStream_t s) {
  PCVL_CHECK(p->forwarded, "pcvl_slos_forward has not run on this plan");
  if (p->B == 1) {
    SlosTiledArgs ta = tiled_args(p, p->n);
    ta.in = p->final_layer();
    const dd inv_in = dd_from_double(1.0 / p->prodfact_in);
    int rc;
    if (p->m <= 8)
      rc = launch_fin_tiled<8>(ta, p->ftail_d, inv_in, mode, w, out_real, out_c, seed, s);
    else if (p->m <= 16)
      rc = launch_fin_tiled<16>(ta, p->ftail_d, inv_in, mode, w, out_real, out_c, seed, s);
    else if (p->m <= 24)
      rc = launch_fin_tiled<24>(ta, p->ftail_d, inv_in, mode, w, out_real, out_c, seed, s);
    else
      rc = launch_fin_tiled<32>(ta, p->ftail_d, inv_in, mode, w, out_real, out_c, seed, s);
    if (rc != 0) {
      set_error("SLOS finalize launch failed: %s", cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
    return PCVL_OK;
  }
  const size_t smem = (size_t)(p->m + 1) * p->cn_stride * sizeof(uint32_t);
  const uint64_t tot = p->sizes[p->n] * (uint64_t)p->B;
  slos_finalize<<<grid_for(tot, 256), 256, smem, s>>>(p->final_layer(), (uint32_t)p->sizes[p->n], p->m, p->n,
                                                      p->B, p->cn_d, p->cn_stride, 1.0 / p->prodfact_in, mode,
                                                      w, out_real, out_c, seed);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}

extern "C" int pcvl_slos_probabilities(pcvl_slos_plan* p, double* probs_d, void* stream) {
  PCVL_CHECK(p && probs_d, "null pointer argument");
  return finalize(p, 0, nullptr, probs_d, nullptr, nullptr, (cudaStream_t)stream);
}

extern "C" int pcvl_slos_amplitudes(pcvl_slos_plan* p, double* amps_d, void* stream) {
  PCVL_CHECK(p && amps_d, "null pointer argument");
  return finalize(p, 1, nullptr, nullptr, (double2*)amps_d, nullptr, (cudaStream_t)stream);
}

extern "C" int pcvl_slos_backward(pcvl_slos_plan* p, const double* weights_d, double* grad_u_d, void* stream_) {
  PCVL_CHECK(p && weights_d && grad_u_d, "null pointer argument");
  PCVL_CHECK(p->keep, "pcvl_slos_backward needs a plan created with keep_layers != 0");
  cudaStream_t s = (cudaStream_t)stream_;
  const int m = p->m, B = p->B, n = p->n;
  PCVL_CUDA(cudaMemsetAsync(grad_u_d, 0, (size_t)B * m * m * 2 * sizeof(double), s));
  PCVL_TRY(finalize(p, 2, weights_d, nullptr, nullptr, p->adj_d[n % 2], s));
  for (int k = n; k >= 1; --k) {
    SlosLayerArgs a{};
    a.m = m;
    a.k = k - 1;  // photons of the parent layer
    a.B = B;
    a.nstates = (uint32_t)p->sizes[k - 1];
    a.in = p->adj_d[k % 2];
    a.out = p->adj_d[(k - 1) % 2];
    const int mk = p->order[k - 1];
    a.ucol = p->ucols_d + (size_t)mk * m * B;
    a.cn = p->cn_d;
    a.cn_stride = p->cn_stride;
    a.cpar = p->layers[k - 1];
    a.gpart = p->gpart_d;
    const int grid = std::min(p->gpart_blocks, B > 1 ? grid_for(a.nstates, 8) : grid_for(a.nstates, 256));
    const int rc = dispatch_layer(true, a, grid, s);
    if (rc != 0) {
      set_error("SLOS adjoint layer %d launch failed: %s", k, cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
    slos_grad_reduce<<<(m * B + 255) / 256, 256, 0, s>>>(p->gpart_d, grid, m, B, mk, (double2*)grad_u_d);
    PCVL_CUDA(cudaGetLastError());
  }
  return PCVL_OK;
}
