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
// Ranks.  Layer k is the k-photon space in descending lexicographic order.  With
// Cn(M, x) = C(M + x - 1, x) (states of x photons on M modes) and R_{i+1} the photons
// in modes after i:
//     rank(s)       = sum_{i <= m-2} Cn(m - i, R_{i+1} - 1)
//     rank(s - e_j) = rank(s) - sum_{i < j} Cn(m - i - 1, R_{i+1}(s) - 1)
//     rank(p + e_j) = rank(p) + sum_{i < j} Cn(m - i - 1, R_{i+1}(p))
//
// Tiles.  The modes split into a prefix (the first p = m - t) and a tail (the last
// t <= 8).  A tile is the set of states sharing one prefix pi; its r = k - |pi| tail
// photons range over the count(t, r) tail states tau, contiguous in rank order:
//     rank(pi, tau) = A(pi, r) + rank_t(tau),   A = sum_{i<p} Cn(m - i, R_{i+1} - 1),
// and tiles are ordered like the states of the (p + 1)-mode space whose last mode
// holds r, so tile index -> pi is one unranking.  From the formulas above:
//   parent through prefix mode j:  A - Pfx_j + tau           Pfx_j = sum_{i<j} Cn(m-i-1, R_{i+1}-1)
//   parent through tail mode j:    A - Pfx_p + TP[r][tau][j] TP = rank_t(tau - e_j)
//   child through prefix mode j:   A + Q_j + tau             Q_j = sum_{i<j} Cn(m-i-1, R_{i+1})
//   child through tail mode j:     A + Q_p + TC[r][tau][j]   TC = rank_t(tau + e_j)
// so a parent or child index costs one add (prefix modes, contiguous over tau) or one
// small-table read (tail modes).  Each lane of a warp computes the descriptor of one
// tile of a group of 32; the warp then sweeps the group's states.
//
// Arithmetic.  Every kernel is instantiated for the two policies of arith.cuh: native
// FP64 (Arith64, the default: complex128 coefficients and DFMA multiply-adds, as the
// reference's complex128 layers) and float-float (ArithFF, opt-in: FP32-pipe pairs,
// ~48 significant bits).  A plan fixes its arithmetic at creation.
//
// Layout.  Coefficients are 16-byte complex values (double2 or a float-float pair),
// state-major with the circuit index b innermost: element (r, b) at r * B + b.  With
// B == 1 the lanes take consecutive states; with B >= 2 the lanes take 32 circuits
// of one state (blockIdx.y selects the 32-circuit chunk), so loads are coalesced
// across circuits and the index work is shared by the 32 lanes.
//
// Batch entries.  Entry b of a plan has its own unitary U_b and its own input state
// (all with the same photon count n: every layer is the same Fock space).  Layer k of
// entry b adds a photon in input mode col[k][b] (its own _Path order), so the layer
// reads u_j(b) = U_b[j, col[k][b]]; the normalisation 1 / prod(in_b!) is per entry.  A
// plan for one input state is the case where every entry has the same columns.
#include <algorithm>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "arith.cuh"
#include "common.cuh"
#include "runtime.cuh"
#include "slos_plan.cuh"

namespace pcvl {

constexpr int kSlosMaxM = 32;
constexpr int kSlosMaxN = 32;
constexpr uint32_t kNone = 0xffffffffu;
constexpr int kWarps = 8;  // warps per CTA (256 threads)
constexpr int kBwdGroups = 2;  // mode groups per warp of the batched adjoint (measured: 2 beats 1 and 4)

// Values (P::V, 16 bytes) and factors (P::F, 8 bytes) travel as untyped pointers; each
// kernel reads them with its arithmetic's types.
struct SlosArgs {
  int m, k, p, t, B;      // k: photons of the layer whose states are the tiles
  uint32_t ntiles;
  const void* in;         // forward: parent layer; adjoint: child-layer adjoint
  void* out;              // forward: child layer; adjoint: parent-layer adjoint
  const void* ucol;       // u_j (b) = U_b[j, mk] at ucol[j * B + b]
  const void* cpar;       // adjoint: forward coefficients of the parent layer
  void* gpart;            // adjoint: per-CTA partials of dL/du_j, [blockIdx.x][j][b]
  const uint32_t* cn;
  int cn_stride;
  const uint32_t* tail;   // TP (forward) or TC (adjoint)
  const void* ftail;      // prod tau_j! per tail state (factors)
  const void* inv_in;     // 1 / prod(in_b!) per batch entry (factors)
  const uint8_t* tocc;    // occupied tail modes per tail state (bit j)
  uint32_t tail_off[kSlosMaxN + 2];    // entry offset of the block of r tail photons
  uint32_t tstate_off[kSlosMaxN + 2];  // state offset of that block
  uint32_t tsize[kSlosMaxN + 2];       // count(t, r)
  // work units of the layer, by tail photon count r (class r: count(p, k - r) tiles
  // of tsize[r] states): unit offsets, tiles, and chunks per tile (0: small tiles,
  // 32 whole tiles per unit, one per lane)
  uint32_t uoff[kSlosMaxN + 2];
  uint32_t npf[kSlosMaxN + 1];
  uint32_t cpt[kSlosMaxN + 1];
  uint32_t chunkB;        // states per unit of the batched kernels
  // units of the single-circuit forward kernel: tiles of >= chunk1 / 2 states (>= chunk1
  // when chunk1 is below its full size) in chunks of chunk1 (cpt1 > 0), smaller tiles in
  // groups of grp1 tiles (about chunk1 states)
  uint32_t chunk1;
  uint32_t uoff1[kSlosMaxN + 2];
  uint32_t cpt1[kSlosMaxN + 1];
  uint32_t grp1[kSlosMaxN + 1];
};

constexpr uint32_t kChunk = 256;   // states per unit of a large tile (single circuit)
constexpr uint32_t kChunkB = 32;   // states per unit (batched forward and finalisation)
constexpr uint32_t kChunkBwdB = 8; // states per unit (batched adjoint: more, smaller units)
constexpr uint32_t kChunk1 = 1024; // largest unit of the single-circuit forward kernel (states)

__device__ __forceinline__ uint32_t cn_at(const uint32_t* cn, int stride, int M, int x) {
  return x < 0 ? 0u : cn[M * stride + x];
}

// Prefix descriptor of one tile, in registers (F: the arithmetic's factor type).
template <int MMAX, typename F>
struct Desc {
  uint32_t A;             // rank of the tile's first state
  uint32_t tb;            // forward: A - Pfx_p; adjoint: A + Q_p
  uint32_t mask;          // occupied prefix modes
  uint32_t base[MMAX];    // forward: A - Pfx_j (occupied j); adjoint: A + Q_j
  F f;                    // prod pi_i! / prod(in!)  (normalisation only)
};

// Unranks prefix pi_idx of the q-photon prefix space (p modes) for a tile with r
// tail photons and walks the modes once for the tile's offsets.
template <int MMAX, bool ADJ, bool FACT, class P>
__device__ __forceinline__ void describe(uint32_t pi_idx, int q, int r, const SlosArgs& a, const uint32_t* cn,
                                         Desc<MMAX, typename P::F>& d, typename P::F inv_in, uint32_t* base) {
  const int m = a.m, p = a.p, st = a.cn_stride;
  uint32_t rho = pi_idx, A = 0, acc = 0, mask = 0;
  int Rp = q, R = q + r;
  typename P::F f = inv_in;
#pragma unroll
  for (int i = 0; i < MMAX; ++i) {
    if (i < p) {
      int v = Rp;
      if (i < p - 1) {
        int x = Rp;
        while (x > 0) {
          const uint32_t c = cn_at(cn, st, p - i, x - 1);
          if (rho >= c) {
            rho -= c;
            break;
          }
          --x;
        }
        v = Rp - x;
      }
      if (FACT)
        for (int s2 = 2; s2 <= v; ++s2) f = P::f_mul_int(f, s2);
      Rp -= v;
      const int Rn = R - v;
      if (ADJ) {
        base[i] = acc;  // Q_i
        acc += cn_at(cn, st, m - i - 1, Rn);
      } else {
        if (v > 0) {
          mask |= 1u << i;
          base[i] = acc;  // Pfx_i
        }
        acc += cn_at(cn, st, m - i - 1, Rn - 1);
      }
      A += cn_at(cn, st, m - i, Rn - 1);
      R = Rn;
    }
  }
#pragma unroll
  for (int i = 0; i < MMAX; ++i) {
    if (i < p) {
      if (ADJ)
        base[i] = A + base[i];
      else if ((mask >> i) & 1u)
        base[i] = A - base[i];
    }
  }
  d.A = A;
  d.tb = ADJ ? A + acc : A - acc;
  d.mask = ADJ ? (p >= 32 ? 0xffffffffu : ((1u << p) - 1u)) : mask;
  if (FACT) d.f = f;
}

// class (tail photon count) of unit u: uniform across the warp
__device__ __forceinline__ int unit_class(const SlosArgs& a, uint32_t u) {
  int r = 0;
  while (r < a.k && a.uoff[r + 1] <= u) ++r;
  return r;
}

// Dynamic shared memory of the layer kernels: [rank table][u].  u holds u_j
// (single circuit, broadcast) or u_j of the CTA's 32 circuits ([j][lane]).
__host__ __device__ inline size_t smem_cn_bytes(int m, int stride) {
  return ((size_t)(m + 1) * stride * sizeof(uint32_t) + 15) / 16 * 16;
}
template <int MMAX>
__host__ __device__ inline size_t smem_bytes(int m, int stride) {
  return smem_cn_bytes(m, stride) + (size_t)MMAX * 32 * sizeof(double2);
}
// rank table and u (conjugated for the adjoint) into shared memory
template <int MMAX, bool BATCHED, bool CONJ, class P>
__device__ __forceinline__ typename P::V* load_shared(const SlosArgs& a, unsigned char* raw, uint32_t*& cn) {
  using V = typename P::V;
  cn = reinterpret_cast<uint32_t*>(raw);
  V* u = reinterpret_cast<V*>(raw + smem_cn_bytes(a.m, a.cn_stride));
  const V* ucol = static_cast<const V*>(a.ucol);
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn[i] = a.cn[i];
  if (BATCHED) {
    for (int i = threadIdx.x; i < MMAX * 32; i += blockDim.x) {
      const int j = i >> 5, b = blockIdx.y * 32 + (i & 31);
      V v = (j < a.m && b < a.B) ? ucol[(size_t)j * a.B + b] : P::zero();
      u[i] = CONJ ? P::conj(v) : v;
    }
  } else if (threadIdx.x < MMAX) {
    V v = (int)threadIdx.x < a.m ? ucol[threadIdx.x] : P::zero();
    u[threadIdx.x] = CONJ ? P::conj(v) : v;
  }
  __syncthreads();
  return u;
}

// Forward value of state (d, tau) with r tail photons for circuit b of a batch: sum over
// its occupied modes of u_j x[parent_j].  Prefix modes follow the tile mask (uniform over
// a tile); tail modes loop over the set bits of the state's own tail occupation.
template <int MMAX, class P>
__device__ __forceinline__ typename P::V fwd_value(const SlosArgs& a, const Desc<MMAX, typename P::F>& d, int r,
                                                   uint32_t tau, const typename P::V* __restrict__ x,
                                                   const typename P::V* u, int us, int b) {
  const int p = a.p;
  typename P::Acc acc = P::acc_zero();
#pragma unroll
  for (int j = 0; j < MMAX; ++j) {
    if (j < p && ((d.mask >> j) & 1u)) {
      const uint32_t ad = d.base[j] + tau;
      P::fma(acc, P::ld(&x[(size_t)ad * a.B + b]), u[j * us]);
    }
  }
  if (r > 0) {
    const uint32_t* row = a.tail + a.tail_off[r] + (size_t)tau * a.t;
    uint32_t occ = __ldg(&a.tocc[a.tstate_off[r] + tau]);  // occupied tail modes
    while (occ) {
      const int jl = __ffs(occ) - 1;
      occ &= occ - 1;
      const uint32_t ad = d.tb + __ldg(&row[jl]);
      P::fma(acc, P::ld(&x[(size_t)ad * a.B + b]), u[(p + jl) * us]);
    }
  }
  return P::finish(acc);
}

// Two consecutive states of one tile for circuit b: the same sums as fwd_value, in the same
// order for each state, as two independent chains (FP64: a complex multiply-add is four
// dependent DFMA per component pair, so one chain per lane leaves the FP64 pipe idle).
template <int MMAX, class P>
__device__ __forceinline__ void fwd_value2(const SlosArgs& a, const Desc<MMAX, typename P::F>& d, int r,
                                           uint32_t tau, bool two, const typename P::V* __restrict__ x,
                                           const typename P::V* u, int b, typename P::V& v0, typename P::V& v1) {
  using V = typename P::V;
  const int p = a.p;
  typename P::Acc acc0 = P::acc_zero(), acc1 = P::acc_zero();
#pragma unroll
  for (int j = 0; j < MMAX; ++j) {
    if (j < p && ((d.mask >> j) & 1u)) {
      const uint32_t ad = d.base[j] + tau;
      const V uj = u[j * 32];
      P::fma(acc0, P::ld(&x[(size_t)ad * a.B + b]), uj);
      if (two) P::fma(acc1, P::ld(&x[(size_t)(ad + 1) * a.B + b]), uj);
    }
  }
  if (r > 0) {
    const uint32_t* row0 = a.tail + a.tail_off[r] + (size_t)tau * a.t;
    uint32_t occ0 = __ldg(&a.tocc[a.tstate_off[r] + tau]);
    uint32_t occ1 = two ? __ldg(&a.tocc[a.tstate_off[r] + tau + 1]) : 0u;
    const uint32_t* row1 = row0 + a.t;
    while (occ0 | occ1) {
      if (occ0) {
        const int jl = __ffs(occ0) - 1;
        occ0 &= occ0 - 1;
        P::fma(acc0, P::ld(&x[(size_t)(d.tb + __ldg(&row0[jl])) * a.B + b]), u[(p + jl) * 32]);
      }
      if (occ1) {
        const int jl = __ffs(occ1) - 1;
        occ1 &= occ1 - 1;
        P::fma(acc1, P::ld(&x[(size_t)(d.tb + __ldg(&row1[jl])) * a.B + b]), u[(p + jl) * 32]);
      }
    }
  }
  v0 = P::finish(acc0);
  v1 = P::finish(acc1);
}

// Batched forward layer: a warp takes a unit (one tile, up to kChunkB states) and its
// lanes 32 circuits; the parent offsets are warp-uniform, the loads coalesced.  In FP64
// a lane carries two states at a time (fwd_value2).
template <int MMAX, class P>
__global__ void __launch_bounds__(256, 4) slos_fwdb(SlosArgs a) {
  using V = typename P::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t* cn;
  const V* us_base = load_shared<MMAX, true, false, P>(a, smem_raw, cn);
  const V* xin = static_cast<const V*>(a.in);
  V* xout = static_cast<V*>(a.out);
  const int lane = threadIdx.x & 31;
  const int b = blockIdx.y * 32 + lane;
  const V* u = us_base + lane;
  const uint32_t total = a.uoff[a.k + 1];
  const uint32_t nw = gridDim.x * kWarps;
  for (uint32_t unit = blockIdx.x * kWarps + (threadIdx.x >> 5); unit < total; unit += nw) {
    const int r = unit_class(a, unit);
    const uint32_t S = a.tsize[r], lu = unit - a.uoff[r], cpt = a.cpt[r];
    const uint32_t pi = lu / cpt, ch = lu - pi * cpt;
    Desc<MMAX, typename P::F> d;
    describe<MMAX, false, false, P>(pi, a.k - r, r, a, cn, d, P::f_from(0.0), d.base);
    const uint32_t t0 = ch * a.chunkB, t1 = min(S, t0 + a.chunkB);
    if (b < a.B) {
      if constexpr (std::is_same<P, Arith64>::value) {
        for (uint32_t tau = t0; tau < t1; tau += 2) {
          const bool two = tau + 1 < t1;
          V v0, v1;
          fwd_value2<MMAX, P>(a, d, r, tau, two, xin, u, b, v0, v1);
          xout[(size_t)(d.A + tau) * a.B + b] = v0;
          if (two) xout[(size_t)(d.A + tau + 1) * a.B + b] = v1;
        }
      } else {
        for (uint32_t tau = t0; tau < t1; ++tau)
          xout[(size_t)(d.A + tau) * a.B + b] = fwd_value<MMAX, P>(a, d, r, tau, xin, u, 32, b);
      }
    }
  }
}

// class of a forward-single unit (uniform across the warp)
__device__ __forceinline__ int unit_class1(const SlosArgs& a, uint32_t u) {
  int r = 0;
  while (r < a.k && a.uoff1[r + 1] <= u) ++r;
  return r;
}

// Words per thread of the single-circuit forward kernel's shared slots: the parent
// offsets of one tile (MMAX), its A, tb and prefix mask, and (probability output) its
// normalisation prod pi! / prod in! as two floats.
template <int MMAX, bool PROB>
__host__ __device__ constexpr int fwd1_slot() {
  return PROB ? MMAX + 5 : MMAX + 4;
}

// Single-circuit forward layer.
//  * Tiles of >= chunk1 / 2 states: a unit is up to chunk1 states of one tile, so the warp shares
//    the tile.  Lane 0 unranks it into its slot; the prefix modes are a warp-uniform loop
//    over the tile's mask (parent offsets and u_j are broadcast reads, parent loads
//    coalesced), then each lane adds its state's tail modes from the tail tables.  A
//    lane takes two states 32 apart per round, so every broadcast read feeds two
//    independent load / multiply-add chains.  (Paired f32x2 forms of the float-float
//    multiply-add were measured slower here: the kernel waits on its gathers.)
//  * Smaller tiles: a unit is a group of grp1 consecutive tiles (about chunk1 states).
//    Lane l unranks tile l of the group into its own slot (all lanes at once), then the
//    warp sweeps the group's states in rank order, one state per lane; each lane loops
//    over the set bits of its state's occupation (prefix bits from its tile's slot, tail
//    bits from the table), so a warp runs as many multiply-adds as its busiest lane.
//  * PROB (the last layer, when only probabilities are wanted): each state's probability
//    |c|^2 prod(out!) / prod(in!) goes to probs instead of its coefficient to a.out, so the
//    last layer is never stored nor read back.
template <int MMAX, bool PROB, class P>
__global__ void __launch_bounds__(256, 6) slos_fwd1(SlosArgs a, double* __restrict__ probs) {
  using V = typename P::V;
  using F = typename P::F;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SL = fwd1_slot<MMAX, PROB>();
  uint32_t* cn;
  const V* u = load_shared<MMAX, false, false, P>(a, smem_raw, cn);
  const V* __restrict__ xin = static_cast<const V*>(a.in);
  V* __restrict__ xout = static_cast<V*>(a.out);
  const F* __restrict__ ftail_all = static_cast<const F*>(a.ftail);
  const F inv0 = PROB ? static_cast<const F*>(a.inv_in)[0] : P::f_from(0.0);
  // one circuit: u holds MMAX entries; the slots follow
  uint32_t* slots = reinterpret_cast<uint32_t*>(smem_raw + smem_cn_bytes(a.m, a.cn_stride) +
                                                (size_t)MMAX * sizeof(V));
  const int lane = threadIdx.x & 31, p = a.p;
  uint32_t* myslot = slots + (size_t)threadIdx.x * SL;
  const uint32_t* wslots = slots + (size_t)(threadIdx.x - lane) * SL;  // the warp's 32 slots
  const uint32_t total = a.uoff1[a.k + 1];
  const uint32_t nw = gridDim.x * kWarps;
  for (uint32_t unit = blockIdx.x * kWarps + (threadIdx.x >> 5); unit < total; unit += nw) {
    const int r = unit_class1(a, unit);
    const int q = a.k - r;
    const uint32_t S = a.tsize[r], lu = unit - a.uoff1[r], cpt = a.cpt1[r];
    const uint8_t* occ_t = a.tocc + a.tstate_off[r];
    const uint32_t* rows = a.tail + a.tail_off[r];
    if (cpt > 0) {  // warp-uniform branch: the class of the unit
      const uint32_t pi = lu / cpt;
      const uint32_t c0 = (lu - pi * cpt) * a.chunk1;
      const uint32_t c1 = min(S, c0 + a.chunk1);
      uint32_t A = 0, tb = 0, mask = 0;
      F ft = P::f_from(0.0);
      if (lane == 0) {
        Desc<MMAX, F> d;
        describe<MMAX, false, PROB, P>(pi, q, r, a, cn, d, inv0, myslot);
        A = d.A;
        tb = d.tb;
        mask = d.mask;
        if (PROB) ft = d.f;
      }
      __syncwarp();
      A = __shfl_sync(0xffffffffu, A, 0);
      tb = __shfl_sync(0xffffffffu, tb, 0);
      mask = __shfl_sync(0xffffffffu, mask, 0);
      if (PROB) ft = P::f_shfl(ft, 0);
      const F* ftail = ftail_all + a.tstate_off[r];
      for (uint32_t t0 = c0 + lane; t0 < c1; t0 += 64) {
        const uint32_t t1 = t0 + 32;
        const bool two = t1 < c1;
        typename P::Acc acc0 = P::acc_zero(), acc1 = P::acc_zero();
        for (uint32_t mm = mask; mm; mm &= mm - 1) {
          const int j = __ffs(mm) - 1;
          const uint32_t bj = wslots[j];
          const V uj = u[j];
          P::fma(acc0, P::ld(&xin[bj + t0]), uj);
          if (two) P::fma(acc1, P::ld(&xin[bj + t1]), uj);
        }
        {
          const uint32_t* row = rows + (size_t)t0 * a.t;
          for (uint32_t o = __ldg(&occ_t[t0]); o; o &= o - 1) {
            const int jl = __ffs(o) - 1;
            P::fma(acc0, P::ld(&xin[tb + __ldg(&row[jl])]), u[p + jl]);
          }
          if (PROB)
            probs[A + t0] = P::prob(P::finish(acc0), P::f_mul(ft, ftail[t0]));
          else
            xout[A + t0] = P::finish(acc0);
        }
        if (two) {
          const uint32_t* row = rows + (size_t)t1 * a.t;
          for (uint32_t o = __ldg(&occ_t[t1]); o; o &= o - 1) {
            const int jl = __ffs(o) - 1;
            P::fma(acc1, P::ld(&xin[tb + __ldg(&row[jl])]), u[p + jl]);
          }
          if (PROB)
            probs[A + t1] = P::prob(P::finish(acc1), P::f_mul(ft, ftail[t1]));
          else
            xout[A + t1] = P::finish(acc1);
        }
      }
      __syncwarp();  // lane 0's slot is rewritten by the next unit
      continue;
    }
    // group of G tiles: lane l unranks tile g0 + l
    const uint32_t G = a.grp1[r];
    const uint32_t g0 = lu * G;
    const uint32_t ng = min(G, a.npf[r] - g0);
    if ((uint32_t)lane < ng) {
      Desc<MMAX, F> d;
      describe<MMAX, false, PROB, P>(g0 + lane, q, r, a, cn, d, inv0, myslot);
      myslot[MMAX] = d.A;
      myslot[MMAX + 1] = d.tb;
      myslot[MMAX + 2] = d.mask;
      if (PROB) P::f_pack(d.f, myslot + MMAX + 3);
    }
    __syncwarp();
    // state f = g * S + tau of the group, f = lane, lane + 32, ...
    const uint32_t q32 = 32 / S, r32 = 32 - q32 * S;
    uint32_t g = (uint32_t)lane / S, tau = (uint32_t)lane - g * S;
    while (g < ng) {
      const uint32_t* ws = wslots + (size_t)g * SL;
      uint32_t occ = ws[MMAX + 2] | ((uint32_t)__ldg(&occ_t[tau]) << p);
      const uint32_t tb = ws[MMAX + 1];
      const uint32_t* row = rows + (size_t)tau * a.t - p;
      typename P::Acc acc = P::acc_zero();
      // two occupied modes per iteration: both parent gathers are in flight before the
      // first multiply-add (the accumulation order, and so the result, is unchanged)
      while (occ) {
        const int j = __ffs(occ) - 1;
        occ &= occ - 1;
        const uint32_t ad = j < p ? ws[j] + tau : tb + __ldg(&row[j]);
        if (occ) {
          const int j2 = __ffs(occ) - 1;
          occ &= occ - 1;
          const uint32_t ad2 = j2 < p ? ws[j2] + tau : tb + __ldg(&row[j2]);
          const V v = P::ld(&xin[ad]), v2 = P::ld(&xin[ad2]);
          P::fma(acc, v, u[j]);
          P::fma(acc, v2, u[j2]);
        } else {
          P::fma(acc, P::ld(&xin[ad]), u[j]);
        }
      }
      if (PROB) {
        const F fg = P::f_unpack(ws + MMAX + 3);
        probs[ws[MMAX] + tau] = P::prob(P::finish(acc), P::f_mul(fg, ftail_all[a.tstate_off[r] + tau]));
      } else {
        xout[ws[MMAX] + tau] = P::finish(acc);
      }
      g += q32;
      tau += r32;
      if (tau >= S) {
        tau -= S;
        ++g;
      }
    }
    __syncwarp();  // the slots are rewritten by the next unit
  }
}

// Adjoint value of parent state (d, tau) of one circuit: a_{k-1} = sum_j conj(u_j)
// a_k[child_j], and g_j += conj(c_{k-1}) a_k[child_j] (every child exists).
template <int MMAX, class P>
__device__ __forceinline__ void bwd_state(const SlosArgs& a, const Desc<MMAX, typename P::F>& d, int r,
                                          uint32_t tau, const typename P::V* uc, typename P::Acc (&g)[MMAX]) {
  using V = typename P::V;
  const int p = a.p, m = a.m;
  const V* __restrict__ xin = static_cast<const V*>(a.in);
  const size_t pidx = (size_t)(d.A + tau);
  const V cp = P::conj(P::ld(&static_cast<const V*>(a.cpar)[pidx]));
  const uint32_t* row = a.tail + a.tail_off[r] + (size_t)tau * a.t;
  typename P::Acc acc = P::acc_zero();
#pragma unroll
  for (int j = 0; j < MMAX; ++j) {
    if (j < m) {
      const uint32_t ad = j < p ? d.base[j] + tau : d.tb + __ldg(&row[j - p]);
      const V v = P::ld(&xin[ad]);
      P::fma(acc, v, uc[j]);
      P::fma(g[j], v, cp);
    }
  }
  static_cast<V*>(a.out)[pidx] = P::finish(acc);
}

// Single-circuit adjoint step over the parent layer (its states are the units' states);
// per-CTA partials of dL/du_j go to gpart.  Batches use slos_bwd_g.
template <int MMAX, class P>
__global__ void __launch_bounds__(256) slos_bwd(SlosArgs a) {
  using V = typename P::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ V red[kWarps][32];
  uint32_t* cn;
  const V* uc = load_shared<MMAX, false, true, P>(a, smem_raw, cn);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int m = a.m;
  typename P::Acc g[MMAX];
#pragma unroll
  for (int j = 0; j < MMAX; ++j) g[j] = P::acc_zero();
  const uint32_t total = a.uoff[a.k + 1];
  const uint32_t nw = gridDim.x * kWarps;
  for (uint32_t unit = blockIdx.x * kWarps + wid; unit < total; unit += nw) {
    const int r = unit_class(a, unit);
    const int q = a.k - r;
    const uint32_t S = a.tsize[r], lu = unit - a.uoff[r], cpt = a.cpt[r];
    Desc<MMAX, typename P::F> d;
    if (cpt > 0) {
      const uint32_t pi = lu / cpt, ch = lu - pi * cpt;
      describe<MMAX, true, false, P>(pi, q, r, a, cn, d, P::f_from(0.0), d.base);
      const uint32_t t0 = ch * kChunk, t1 = min(S, t0 + kChunk);
      for (uint32_t tau = t0 + lane; tau < t1; tau += 32) bwd_state<MMAX, P>(a, d, r, tau, uc, g);
    } else {
      // small tiles: one tile per lane
      const uint32_t pi = lu * 32 + lane;
      if (pi < a.npf[r]) {
        describe<MMAX, true, false, P>(pi, q, r, a, cn, d, P::f_from(0.0), d.base);
        for (uint32_t tau = 0; tau < S; ++tau) bwd_state<MMAX, P>(a, d, r, tau, uc, g);
      }
    }
  }
  // reduce g over the CTA's threads
  V* gpart = static_cast<V*>(a.gpart);
#pragma unroll
  for (int j = 0; j < MMAX; ++j) {
    if (j >= m) break;
    V v = P::finish(g[j]);
#pragma unroll
    for (int dlt = 16; dlt > 0; dlt >>= 1) v = P::add(v, P::shfl_down(v, dlt));
    red[wid][lane] = v;
    __syncthreads();
    if (wid == 0 && lane == 0) {
      V s2 = red[0][0];
      for (int w = 1; w < kWarps; ++w) s2 = P::add(s2, red[w][0]);
      gpart[(size_t)blockIdx.x * m + j] = s2;
    }
    __syncthreads();
  }
}


// Batched adjoint with a fraction of the accumulator registers: the lanes of a warp are
// G mode groups x 32/G circuits.  Lane l serves circuit blockIdx.y * 32/G + l % (32/G) for
// the modes j = (l / (32/G)) * MMAX/G + jj, so it keeps the float-float partials of
// dL/du_j for MMAX/G modes; the G group parts of a parent's
// a_{k-1} = sum_j conj(u_j) a_k[child_j] meet by log2(G) shuffles.  Every (parent, mode,
// circuit) child value is loaded once, as in slos_bwd.
template <int MMAX, int G, class P>
__global__ void __launch_bounds__(256, MMAX <= 16 ? 4 : 2) slos_bwd_g(SlosArgs a) {
  using V = typename P::V;
  constexpr int NC = 32 / G, MG = MMAX / G;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ V red[kWarps][32];
  uint32_t* cn = reinterpret_cast<uint32_t*>(smem_raw);
  V* us = reinterpret_cast<V*>(smem_raw + smem_cn_bytes(a.m, a.cn_stride));  // [j][NC circuits], conjugated
  const V* ucol = static_cast<const V*>(a.ucol);
  const V* __restrict__ xin = static_cast<const V*>(a.in);
  const V* __restrict__ cpar = static_cast<const V*>(a.cpar);
  V* __restrict__ xout = static_cast<V*>(a.out);
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn[i] = a.cn[i];
  for (int i = threadIdx.x; i < MMAX * NC; i += blockDim.x) {
    const int j = i / NC, b = blockIdx.y * NC + (i % NC);
    us[i] = (j < a.m && b < a.B) ? P::conj(ucol[(size_t)j * a.B + b]) : P::zero();
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int cl = lane % NC, grp = lane / NC;
  const int b = blockIdx.y * NC + cl;
  const bool live = b < a.B;
  const int m = a.m, p = a.p;
  typename P::Acc g[MG];
#pragma unroll
  for (int jj = 0; jj < MG; ++jj) g[jj] = P::acc_zero();
  const uint32_t total = a.uoff[a.k + 1];
  const uint32_t nw = gridDim.x * kWarps;
  for (uint32_t unit = blockIdx.x * kWarps + wid; unit < total; unit += nw) {
    const int r = unit_class(a, unit);
    const int q = a.k - r;
    const uint32_t S = a.tsize[r], lu = unit - a.uoff[r], cpt = a.cpt[r];
    Desc<MMAX, typename P::F> d;
    const uint32_t pi = lu / cpt, ch = lu - pi * cpt;
    describe<MMAX, true, false, P>(pi, q, r, a, cn, d, P::f_from(0.0), d.base);
    const uint32_t t0 = ch * a.chunkB, t1 = min(S, t0 + a.chunkB);
    for (uint32_t tau = t0; tau < t1; ++tau) {
      const size_t pidx = (size_t)(d.A + tau) * a.B + b;
      const V cp = live ? P::conj(P::ld(&cpar[pidx])) : P::zero();
      const uint32_t* row = a.tail + a.tail_off[r] + (size_t)tau * a.t;
      typename P::Acc acc = P::acc_zero();
#pragma unroll
      for (int jj = 0; jj < MG; ++jj) {
        const int j = grp * MG + jj;
        if (j < m && live) {
          const uint32_t ad = j < p ? d.base[j] + tau : d.tb + __ldg(&row[j - p]);
          const V v = P::ld(&xin[(size_t)ad * a.B + b]);
          P::fma(acc, v, us[j * NC + cl]);
          P::fma(g[jj], v, cp);
        }
      }
      V part = P::finish(acc);
#pragma unroll
      for (int dl = NC; dl < 32; dl <<= 1) part = P::add(part, P::shfl_xor(part, dl));
      if (grp == 0 && live) xout[pidx] = part;
    }
  }
  // per-CTA partials: lane l holds mode (l / NC) * MG + jj of circuit l % NC
  V* gpart = static_cast<V*>(a.gpart);
#pragma unroll
  for (int jj = 0; jj < MG; ++jj) {
    red[wid][lane] = P::finish(g[jj]);
    __syncthreads();
    if (wid == 0) {
      V s2 = red[0][lane];
      for (int w = 1; w < kWarps; ++w) s2 = P::add(s2, red[w][lane]);
      const int j = grp * MG + jj;
      if (j < m && live) gpart[((size_t)blockIdx.x * m + j) * a.B + b] = s2;
    }
    __syncthreads();
  }
}

// Last layer -> probabilities (mode 0), amplitudes (mode 1) or the adjoint seed
// a_n = 2 w F c_n (mode 2), with F = prod(out!) / prod(in!) = f(tile) x ftail[tau].
template <class P>
__device__ __forceinline__ void fin_state(const SlosArgs& a, typename P::F f, int r, size_t idx, int mode,
                                          const double* __restrict__ w_in, double* __restrict__ out_real,
                                          double2* __restrict__ out_c, void* __restrict__ seed, uint32_t tau) {
  using V = typename P::V;
  const typename P::F F = P::f_mul(f, static_cast<const typename P::F*>(a.ftail)[a.tstate_off[r] + tau]);
  const V c = P::ld(&static_cast<const V*>(a.in)[idx]);
  if (mode == 0)
    out_real[idx] = P::prob(c, F);
  else if (mode == 1)
    out_c[idx] = P::amp(c, F);
  else
    static_cast<V*>(seed)[idx] = P::seed(c, w_in[idx], F);
}

template <int MMAX, class P>
__global__ void __launch_bounds__(256) slos_fin(SlosArgs a, int mode, const double* __restrict__ w_in,
                                               double* __restrict__ out_real, double2* __restrict__ out_c,
                                               void* __restrict__ seed) {
  using F = typename P::F;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t* cn = reinterpret_cast<uint32_t*>(smem_raw);
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn[i] = a.cn[i];
  __syncthreads();
  const F* inv_in = static_cast<const F*>(a.inv_in);
  const F one = P::f_from(1.0);
  const int lane = threadIdx.x & 31;
  const bool batched = a.B > 1;
  const int b = batched ? blockIdx.y * 32 + lane : 0;
  const uint32_t total = a.uoff[a.k + 1];
  const uint32_t nw = gridDim.x * kWarps;
  for (uint32_t unit = blockIdx.x * kWarps + (threadIdx.x >> 5); unit < total; unit += nw) {
    const int r = unit_class(a, unit);
    const int q = a.k - r;
    const uint32_t S = a.tsize[r], lu = unit - a.uoff[r], cpt = a.cpt[r];
    Desc<MMAX, F> d;
    if (cpt > 0) {
      const uint32_t pi = lu / cpt, ch = lu - pi * cpt;
      describe<MMAX, false, true, P>(pi, q, r, a, cn, d, one, d.base);
      const uint32_t chunk = batched ? a.chunkB : kChunk;
      const uint32_t t0 = ch * chunk, t1 = min(S, t0 + chunk);
      if (batched) {
        if (b < a.B) {
          const F fb = P::f_mul(d.f, inv_in[b]);
          for (uint32_t tau = t0; tau < t1; ++tau)
            fin_state<P>(a, fb, r, (size_t)(d.A + tau) * a.B + b, mode, w_in, out_real, out_c, seed, tau);
        }
      } else {
        const F fb = P::f_mul(d.f, inv_in[0]);
        for (uint32_t tau = t0 + lane; tau < t1; tau += 32)
          fin_state<P>(a, fb, r, d.A + tau, mode, w_in, out_real, out_c, seed, tau);
      }
    } else {
      const uint32_t pi = lu * 32 + lane;
      if (pi < a.npf[r]) {
        describe<MMAX, false, true, P>(pi, q, r, a, cn, d, one, d.base);
        const F fb = P::f_mul(d.f, inv_in[0]);
        for (uint32_t tau = 0; tau < S; ++tau)
          fin_state<P>(a, fb, r, d.A + tau, mode, w_in, out_real, out_c, seed, tau);
      }
    }
  }
}

// Single-circuit finalisation over the forward kernel's units (uoff1 / cpt1 / grp1):
// large tiles in chunks with one unranking per unit (lane 0, broadcast), smaller tiles
// in groups unranked by all lanes at once and swept in rank order, one state per lane.
template <int MMAX, class P>
__global__ void __launch_bounds__(256) slos_fin1(SlosArgs a, int mode, const double* __restrict__ w_in,
                                                double* __restrict__ out_real, double2* __restrict__ out_c,
                                                void* __restrict__ seed) {
  using F = typename P::F;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t* cn = reinterpret_cast<uint32_t*>(smem_raw);
  const int ncn = (a.m + 1) * a.cn_stride;
  for (int i = threadIdx.x; i < ncn; i += blockDim.x) cn[i] = a.cn[i];
  // per thread: A and the two words of the factor of the tile it unranked
  uint32_t* slots = reinterpret_cast<uint32_t*>(smem_raw + smem_cn_bytes(a.m, a.cn_stride));
  __syncthreads();
  const int lane = threadIdx.x & 31;
  uint32_t* myslot = slots + (size_t)threadIdx.x * 4;
  const uint32_t* wslots = slots + (size_t)(threadIdx.x - lane) * 4;
  const F inv0 = static_cast<const F*>(a.inv_in)[0];
  const uint32_t total = a.uoff1[a.k + 1];
  const uint32_t nw = gridDim.x * kWarps;
  for (uint32_t unit = blockIdx.x * kWarps + (threadIdx.x >> 5); unit < total; unit += nw) {
    const int r = unit_class1(a, unit);
    const int q = a.k - r;
    const uint32_t S = a.tsize[r], lu = unit - a.uoff1[r], cpt = a.cpt1[r];
    if (cpt > 0) {
      const uint32_t pi = lu / cpt;
      const uint32_t c0 = (lu - pi * cpt) * a.chunk1;
      const uint32_t c1 = min(S, c0 + a.chunk1);
      uint32_t A = 0;
      F f = P::f_from(0.0);
      if (lane == 0) {
        Desc<MMAX, F> d;
        describe<MMAX, false, true, P>(pi, q, r, a, cn, d, inv0, d.base);
        A = d.A;
        f = d.f;
      }
      A = __shfl_sync(0xffffffffu, A, 0);
      f = P::f_shfl(f, 0);
      for (uint32_t tau = c0 + lane; tau < c1; tau += 32)
        fin_state<P>(a, f, r, A + tau, mode, w_in, out_real, out_c, seed, tau);
      continue;
    }
    const uint32_t G = a.grp1[r];
    const uint32_t g0 = lu * G;
    const uint32_t ng = min(G, a.npf[r] - g0);
    if ((uint32_t)lane < ng) {
      Desc<MMAX, F> d;
      describe<MMAX, false, true, P>(g0 + lane, q, r, a, cn, d, inv0, d.base);
      myslot[0] = d.A;
      P::f_pack(d.f, myslot + 1);
    }
    __syncwarp();
    const uint32_t q32 = 32 / S, r32 = 32 - q32 * S;
    uint32_t g = (uint32_t)lane / S, tau = (uint32_t)lane - g * S;
    while (g < ng) {
      const uint32_t* ws = wslots + (size_t)g * 4;
      fin_state<P>(a, P::f_unpack(ws + 1), r, ws[0] + tau, mode, w_in, out_real, out_c, seed, tau);
      g += q32;
      tau += r32;
      if (tau >= S) {
        tau -= S;
        ++g;
      }
    }
    __syncwarp();  // the slots are rewritten by the next unit
  }
}

// grad[b][j][col[b]] += sum over CTAs of gpart[cta][j][b]  (col: the layer's column per entry)
template <class P>
__global__ void slos_grad_reduce(const typename P::V* __restrict__ gpart, int nblk, int m, int B,
                                 const int32_t* __restrict__ col, double2* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // i = j * B + b
  if (i >= m * B) return;
  const int j = i / B, b = i - j * B;
  typename P::V s = P::zero();
  for (int q = 0; q < nblk; ++q) s = P::add(s, gpart[(size_t)q * m * B + i]);
  double2* g = &grad[((size_t)b * m + j) * m + col[b]];
  g->x += P::re(s);
  g->y += P::im(s);
}

// ucols[k][j][b] = U_b[j][col[k][b]] in the plan's arithmetic, for the n layers (ustride:
// elements between consecutive entries' unitaries; 0 = one unitary shared by every entry)
template <class P>
__global__ void slos_convert_u(const double2* __restrict__ u, int m, int n, int B, size_t ustride,
                               const int32_t* __restrict__ col, typename P::V* __restrict__ ucols) {
  const size_t tot = (size_t)n * m * B;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
    const size_t kj = i / B;
    const int b = (int)(i - kj * B);
    const int k = (int)(kj / m), j = (int)(kj - (size_t)k * m);
    const double2 v = u[(size_t)b * ustride + (size_t)j * m + col[(size_t)k * B + b]];
    ucols[i] = P::from(v.x, v.y);
  }
}

template <class P>
__global__ void slos_fill_vacuum(typename P::V* layer0, int B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < B) layer0[b] = P::one();
}

enum class Kern { Fwd, FwdProb, Bwd, Fin };

template <int MMAX, class P>
static int launch_kernel(Kern kind, const SlosArgs& a, int grid, int mode, const double* w, double* out_real,
                         double2* out_c, void* seed, cudaStream_t s) {
  using V = typename P::V;
  const size_t smem = smem_bytes<MMAX>(a.m, a.cn_stride);
  const bool batched = a.B > 1;
  dim3 g(grid, batched ? (a.B + 31) / 32 : 1);
  // the descriptors of 8 warps, u and the rank table may pass 48 KB: allow it
  cudaFuncSetAttribute(slos_fwdb<MMAX, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(slos_bwd<MMAX, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(slos_fin<MMAX, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  switch (kind) {
    case Kern::Fwd:
      if (batched) {
        slos_fwdb<MMAX, P><<<g, 256, smem, s>>>(a);
      } else {
        const size_t smem1 = smem_cn_bytes(a.m, a.cn_stride) + (size_t)MMAX * sizeof(V) +
                             (size_t)256 * fwd1_slot<MMAX, false>() * sizeof(uint32_t);
        cudaFuncSetAttribute(slos_fwd1<MMAX, false, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
        slos_fwd1<MMAX, false, P><<<g, 256, smem1, s>>>(a, nullptr);
      }
      break;
    case Kern::FwdProb: {  // single circuit only
      const size_t smem1 = smem_cn_bytes(a.m, a.cn_stride) + (size_t)MMAX * sizeof(V) +
                           (size_t)256 * fwd1_slot<MMAX, true>() * sizeof(uint32_t);
      cudaFuncSetAttribute(slos_fwd1<MMAX, true, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
      slos_fwd1<MMAX, true, P><<<g, 256, smem1, s>>>(a, out_real);
      break;
    }
    case Kern::Bwd:
      if (batched) {
        constexpr int G = kBwdGroups;
        const dim3 gh(grid, (a.B + 32 / G - 1) / (32 / G));
        const size_t smemh = smem_cn_bytes(a.m, a.cn_stride) + (size_t)MMAX * (32 / G) * sizeof(V);
        slos_bwd_g<MMAX, G, P><<<gh, 256, smemh, s>>>(a);
      } else {
        slos_bwd<MMAX, P><<<g, 256, smem, s>>>(a);
      }
      break;
    case Kern::Fin:
      if (batched) {
        slos_fin<MMAX, P><<<g, 256, smem, s>>>(a, mode, w, out_real, out_c, seed);
      } else {
        const size_t smemf = smem_cn_bytes(a.m, a.cn_stride) + (size_t)256 * 4 * sizeof(uint32_t);
        slos_fin1<MMAX, P><<<g, 256, smemf, s>>>(a, mode, w, out_real, out_c, seed);
      }
      break;
  }
  return (int)cudaGetLastError();
}

template <class P>
static int dispatch_p(Kern kind, const SlosArgs& a, int grid, cudaStream_t s, int mode, const double* w,
                      double* out_real, double2* out_c, void* seed) {
  if (a.m <= 8) return launch_kernel<8, P>(kind, a, grid, mode, w, out_real, out_c, seed, s);
  if (a.m <= 16) return launch_kernel<16, P>(kind, a, grid, mode, w, out_real, out_c, seed, s);
  if (a.m <= 24) return launch_kernel<24, P>(kind, a, grid, mode, w, out_real, out_c, seed, s);
  return launch_kernel<32, P>(kind, a, grid, mode, w, out_real, out_c, seed, s);
}

static int dispatch(int prec, Kern kind, const SlosArgs& a, int grid, cudaStream_t s, int mode = 0,
                    const double* w = nullptr, double* out_real = nullptr, double2* out_c = nullptr,
                    void* seed = nullptr) {
  if (prec == kPrecFP64) return dispatch_p<Arith64>(kind, a, grid, s, mode, w, out_real, out_c, seed);
  return dispatch_p<ArithFF>(kind, a, grid, s, mode, w, out_real, out_c, seed);
}

}  // namespace pcvl

using namespace pcvl;

namespace {

void free_plan(pcvl_slos_plan* p) {
  if (!p) return;
  cudaFree(p->cn_d);
  cudaFree(p->col_d);
  cudaFree(p->inv_in_d);
  cudaFree(p->ucols_d);
  for (cdd* l : p->layers) cudaFree(l);
  cudaFree(p->adj_d[0]);
  cudaFree(p->adj_d[1]);
  cudaFree(p->gpart_d);
  cudaFree(p->tp_d);
  cudaFree(p->tc_d);
  cudaFree(p->tocc_d);
  cudaFree(p->ftail_d);
  slos_masked_free(p);
  delete p;
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

uint32_t tail_rank(int t, const std::vector<int>& s) {
  int rest = 0;
  for (int v : s) rest += v;
  uint64_t r = 0;
  for (int i = 0; i < t; ++i) {
    rest -= s[i];
    if (rest > 0) r += fock_count(t - i, rest - 1);
  }
  return (uint32_t)r;
}

// Tail tables for t tail modes and 0..n tail photons (descending-lex order within each
// photon number): parent ranks rank_t(tau - e_j) (kNone where tau_j = 0), child ranks
// rank_t(tau + e_j), and the factorial products prod_j tau_j!.
void tail_tables(int t, int n, std::vector<uint32_t>& tp, std::vector<uint32_t>& tc, std::vector<double>& ftail,
                 std::vector<uint8_t>& tocc, std::vector<uint32_t>& tail_off, std::vector<uint32_t>& tstate_off,
                 std::vector<uint32_t>& tsize) {
  tail_off.assign(n + 2, 0);
  tstate_off.assign(n + 2, 0);
  tsize.assign(n + 2, 0);
  tp.clear();
  tc.clear();
  ftail.clear();
  tocc.clear();
  for (int r = 0; r <= n + 1; ++r) {
    tail_off[r] = (uint32_t)tp.size();
    tstate_off[r] = (uint32_t)ftail.size();
    tsize[r] = (uint32_t)fock_count(t, r);
    if (r > n) break;
    std::vector<int> s(t, 0);
    s[0] = r;
    for (uint32_t q = 0; q < tsize[r]; ++q) {
      double f = 1.0;
      uint8_t occ = 0;
      for (int j = 0; j < t; ++j) {
        if (s[j] > 0) occ |= (uint8_t)(1u << j);
        for (int v = 2; v <= s[j]; ++v) f *= v;
        if (s[j] == 0) {
          tp.push_back(kNone);
        } else {
          s[j] -= 1;
          tp.push_back(tail_rank(t, s));
          s[j] += 1;
        }
        s[j] += 1;
        tc.push_back(tail_rank(t, s));
        s[j] -= 1;
      }
      ftail.push_back(f);
      tocc.push_back(occ);
      int tail = 0;  // next state in descending-lex order
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
}

// factors of the plan's arithmetic as 8-byte words: dd (float-float) or double (FP64)
std::vector<uint64_t> factor_words(const std::vector<double>& x, int prec) {
  std::vector<uint64_t> w(x.size());
  for (size_t i = 0; i < x.size(); ++i) {
    if (prec == kPrecFP64) {
      memcpy(&w[i], &x[i], 8);
    } else {
      const dd v = dd_from_double(x[i]);
      memcpy(&w[i], &v, 8);
    }
  }
  return w;
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

int upload(void* dst, const void* src, size_t bytes) {
  if (cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    pcvl::set_error("SLOS plan: table upload failed");
    return PCVL_ERR_CUDA;
  }
  return PCVL_OK;
}

SlosArgs make_args(const pcvl_slos_plan* p, int k, uint32_t chunkB = kChunkB) {
  SlosArgs a{};
  a.chunkB = chunkB;
  a.m = p->m;
  a.k = k;
  a.p = p->tail_p;
  a.t = p->tail_t;
  a.B = p->B;
  a.ntiles = (uint32_t)fock_count(p->tail_p + 1, k);
  a.cn = p->cn_d;
  a.cn_stride = p->cn_stride;
  a.ftail = p->ftail_d;
  a.inv_in = p->inv_in_d;
  a.tocc = p->tocc_d;
  for (int r = 0; r <= p->n + 1; ++r) {
    a.tail_off[r] = p->tail_off[r];
    a.tstate_off[r] = p->tstate_off[r];
    a.tsize[r] = p->tsize[r];
  }
  // work units by class r = tail photons: batched -> (tile, chunkB states); single
  // circuit -> (tile, kChunk states) for tiles of >= 32 states, 32 whole tiles below
  uint64_t u = 0;
  for (int r = 0; r <= k; ++r) {
    const uint64_t npf = fock_count(p->tail_p, k - r), S = p->tsize[r];
    a.uoff[r] = (uint32_t)u;
    a.npf[r] = (uint32_t)npf;
    if (p->B > 1) {
      a.cpt[r] = (uint32_t)((S + chunkB - 1) / chunkB);
      u += npf * a.cpt[r];
    } else if (S >= 32) {
      a.cpt[r] = (uint32_t)((S + kChunk - 1) / kChunk);
      u += npf * a.cpt[r];
    } else {
      a.cpt[r] = 0;
      u += (npf + 31) / 32;
    }
  }
  a.uoff[k + 1] = (uint32_t)u;
  // unit size: kChunk1 states, smaller (down to 64) when the layer would not give every
  // resident warp several units
  uint64_t chunk = kChunk1;
  const uint64_t want_units = (uint64_t)pcvl::num_sms() * 64;
  while (chunk > 64 && fock_count(p->m, k) / chunk < want_units) chunk >>= 1;
  a.chunk1 = (uint32_t)chunk;
  // tiles of at least half a full unit are units of their own (the warp-uniform path);
  // measured at m = 24, n = 12: half a unit 41.96 ms, a whole unit 42.35, a quarter 42.67,
  // an eighth 45.18 (probabilities of every output), identical results
  const uint64_t big = chunk >= kChunk1 ? chunk / 2 : chunk;
  uint64_t u1 = 0;
  for (int r = 0; r <= k; ++r) {
    const uint64_t npf = fock_count(p->tail_p, k - r), S = p->tsize[r];
    a.uoff1[r] = (uint32_t)u1;
    if (S >= big) {
      a.cpt1[r] = (uint32_t)((S + chunk - 1) / chunk);
      a.grp1[r] = 0;
      u1 += npf * a.cpt1[r];
    } else {
      a.cpt1[r] = 0;
      a.grp1[r] = (uint32_t)std::min<uint64_t>(32, std::max<uint64_t>(1, chunk / S));
      u1 += (npf + a.grp1[r] - 1) / a.grp1[r];
    }
  }
  a.uoff1[k + 1] = (uint32_t)u1;
  return a;
}

// CTAs for a layer: one warp per unit, capped at 16 CTAs per SM (grid-stride beyond)
int grid_for_units(const SlosArgs& a, bool fwd1 = false) {
  const uint64_t units = fwd1 ? a.uoff1[a.k + 1] : a.uoff[a.k + 1];
  uint64_t g = (units + kWarps - 1) / kWarps;
  g = std::min<uint64_t>(g, (uint64_t)pcvl::num_sms() * 16);
  return (int)std::max<uint64_t>(g, 1);
}

}  // namespace

int pcvl::slos_alloc(void** p, size_t bytes, int64_t& total) { return alloc(p, bytes, total); }
int pcvl::slos_upload(void* dst, const void* src, size_t bytes) { return upload(dst, src, bytes); }
std::vector<uint64_t> pcvl::slos_factor_words(const std::vector<double>& x, int prec) {
  return factor_words(x, prec);
}
std::vector<int> pcvl::slos_path_order(const std::vector<int>& input) { return path_order(input); }
void pcvl::slos_free_plan(pcvl_slos_plan* p) { free_plan(p); }

// Plan for `batch` entries with input states inputs[b * m .. b * m + m - 1].
static int create_plan(pcvl_slos_plan** plan, int32_t m, const int32_t* inputs, int32_t batch, int32_t keep_layers,
                       int32_t precision) {
  PCVL_CHECK(plan && inputs, "null pointer argument");
  *plan = nullptr;
  PCVL_CHECK(precision == kPrecFP64 || precision == kPrecFloatFloat,
             "precision must be %d (FP64) or %d (float-float), got %d", (int)kPrecFP64, (int)kPrecFloatFloat,
             precision);
  PCVL_CHECK(m >= 1 && m <= kSlosMaxM, "m=%d outside [1, %d]", m, kSlosMaxM);
  PCVL_CHECK(batch >= 1, "batch must be >= 1");
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
  PCVL_CHECK(n <= kSlosMaxN, "n=%d photons exceeds %d", n, kSlosMaxN);

  auto* p = new (std::nothrow) pcvl_slos_plan();
  PCVL_CHECK(p, "host allocation failed");
  p->m = m;
  p->n = n;
  p->B = batch;
  p->prec = precision;
  p->keep = keep_layers != 0;
  p->inputs.assign(inputs, inputs + (size_t)batch * m);
  p->col.assign((size_t)std::max(n, 1) * batch, 0);
  std::vector<double> inv_in_v(batch);
  for (int b = 0; b < batch; ++b) {
    const std::vector<int> in(inputs + (size_t)b * m, inputs + (size_t)(b + 1) * m);
    const std::vector<int> order = path_order(in);
    for (int k = 0; k < n; ++k) p->col[(size_t)k * batch + b] = order[k];
    double f = 1.0;
    for (int i = 0; i < m; ++i)
      for (int v = 2; v <= in[i]; ++v) f *= v;
    inv_in_v[b] = 1.0 / f;
  }
  const std::vector<uint64_t> inv_in = factor_words(inv_in_v, precision);
  p->sizes.resize(n + 1);
  for (int k = 0; k <= n; ++k) {
    p->sizes[k] = fock_count(m, k);
    if (p->sizes[k] >= 0xffffffffull) {
      delete p;
      set_error("SLOS layer %d holds %llu states: more than 2^32 - 1 states per layer is not supported", k,
                (unsigned long long)fock_count(m, k));
      return PCVL_ERR_ARG;
    }
  }
  // predicted footprint, refused before any allocation
  const size_t B = (size_t)batch;
  size_t need = 0;
  if (p->keep) {
    size_t mx = 0;
    for (int k = 0; k <= n; ++k) {
      need += p->sizes[k] * B * sizeof(cdd);
      mx = std::max<size_t>(mx, p->sizes[k]);
    }
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
  // the tail: at most 8 modes and a table of at most 10^6 tail states over 0..n+1 photons
  int t = std::min(m, 8);
  while (t > 1 && fock_count(t + 1, n + 1) > 1000000ull) --t;
  p->tail_t = t;
  p->tail_p = m - t;
  std::vector<uint32_t> tp, tc;
  std::vector<double> ftail_v;
  std::vector<uint8_t> tocc;
  tail_tables(t, n, tp, tc, ftail_v, tocc, p->tail_off, p->tstate_off, p->tsize);
  const std::vector<uint64_t> ftail = factor_words(ftail_v, precision);
  p->cn_stride = n + 2;
  std::vector<uint32_t> cn((size_t)(m + 1) * p->cn_stride);
  for (int M = 0; M <= m; ++M)
    for (int x = 0; x < p->cn_stride; ++x) {
      const uint64_t v = fock_count(M, x);
      cn[(size_t)M * p->cn_stride + x] = v > 0xffffffffull ? 0xffffffffu : (uint32_t)v;
    }
  if ((rc = alloc((void**)&p->cn_d, cn.size() * 4, p->bytes)) != PCVL_OK) goto fail;
  if ((rc = upload(p->cn_d, cn.data(), cn.size() * 4)) != PCVL_OK) goto fail;
  if ((rc = alloc((void**)&p->tp_d, tp.size() * 4, p->bytes)) != PCVL_OK) goto fail;
  if ((rc = upload(p->tp_d, tp.data(), tp.size() * 4)) != PCVL_OK) goto fail;
  if ((rc = alloc((void**)&p->tc_d, tc.size() * 4, p->bytes)) != PCVL_OK) goto fail;
  if ((rc = upload(p->tc_d, tc.data(), tc.size() * 4)) != PCVL_OK) goto fail;
  if ((rc = alloc((void**)&p->tocc_d, tocc.size(), p->bytes)) != PCVL_OK) goto fail;
  if ((rc = upload(p->tocc_d, tocc.data(), tocc.size())) != PCVL_OK) goto fail;
  if ((rc = alloc((void**)&p->ftail_d, ftail.size() * 8, p->bytes)) != PCVL_OK) goto fail;
  if ((rc = upload(p->ftail_d, ftail.data(), ftail.size() * 8)) != PCVL_OK) goto fail;
  if ((rc = alloc((void**)&p->col_d, p->col.size() * 4, p->bytes)) != PCVL_OK) goto fail;
  if ((rc = upload(p->col_d, p->col.data(), p->col.size() * 4)) != PCVL_OK) goto fail;
  if ((rc = alloc((void**)&p->inv_in_d, B * 8, p->bytes)) != PCVL_OK) goto fail;
  if ((rc = upload(p->inv_in_d, inv_in.data(), B * 8)) != PCVL_OK) goto fail;
  if ((rc = alloc((void**)&p->ucols_d, (size_t)std::max(n, 1) * m * B * sizeof(cdd), p->bytes)) != PCVL_OK)
    goto fail;
  if (p->keep) {
    p->layers.assign(n + 1, nullptr);
    for (int k = 0; k <= n; ++k)
      if ((rc = alloc((void**)&p->layers[k], p->sizes[k] * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
    size_t mx = 0;
    for (int k = 0; k <= n; ++k) mx = std::max<size_t>(mx, p->sizes[k]);
    for (int i = 0; i < 2; ++i)
      if ((rc = alloc((void**)&p->adj_d[i], mx * B * sizeof(cdd), p->bytes)) != PCVL_OK) goto fail;
    p->gpart_blocks = pcvl::num_sms() * 16;
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
  *plan = p;
  return PCVL_OK;
fail:
  free_plan(p);
  return rc;
}

extern "C" int pcvl_slos_plan_create(pcvl_slos_plan** plan, int32_t m, const int32_t* input_state_h,
                                     int32_t batch, int32_t keep_layers, int32_t precision) {
  PCVL_CHECK(plan && input_state_h, "null pointer argument");
  PCVL_CHECK(m >= 1 && m <= kSlosMaxM, "m=%d outside [1, %d]", m, kSlosMaxM);
  PCVL_CHECK(batch >= 1, "batch must be >= 1");
  std::vector<int32_t> inputs((size_t)batch * m);
  for (int b = 0; b < batch; ++b) std::copy(input_state_h, input_state_h + m, inputs.begin() + (size_t)b * m);
  return create_plan(plan, m, inputs.data(), batch, keep_layers, precision);
}

extern "C" int pcvl_slos_plan_create_multi(pcvl_slos_plan** plan, int32_t m, const int32_t* input_states_h,
                                           int32_t batch, int32_t keep_layers, int32_t precision) {
  return create_plan(plan, m, input_states_h, batch, keep_layers, precision);
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

// probs != nullptr (one circuit, full space, n >= 1): the last layer writes probabilities
// instead of coefficients and the plan's last layer is left unwritten.
static int forward(pcvl_slos_plan* p, const double* u_d, size_t ustride, cudaStream_t s, double* probs = nullptr) {
  const int m = p->m, B = p->B;
  if (p->n > 0) {
    const uint64_t tot = (uint64_t)p->n * m * B;
    const int g = (int)std::max<uint64_t>(1, std::min<uint64_t>((tot + 255) / 256, 4096));
    if (p->prec == kPrecFP64)
      slos_convert_u<Arith64><<<g, 256, 0, s>>>((const double2*)u_d, m, p->n, B, ustride, p->col_d,
                                                (double2*)p->ucols_d);
    else
      slos_convert_u<ArithFF><<<g, 256, 0, s>>>((const double2*)u_d, m, p->n, B, ustride, p->col_d, p->ucols_d);
  }
  PCVL_CUDA(cudaGetLastError());
  if (p->prec == kPrecFP64)
    slos_fill_vacuum<Arith64><<<(B + 255) / 256, 256, 0, s>>>((double2*)p->layers[0], B);
  else
    slos_fill_vacuum<ArithFF><<<(B + 255) / 256, 256, 0, s>>>(p->layers[0], B);
  PCVL_CUDA(cudaGetLastError());
  if (p->masked) {
    PCVL_TRY(slos_masked_forward(p, s));
    p->forwarded = true;
    return PCVL_OK;
  }
  for (int k = 1; k <= p->n; ++k) {
    SlosArgs a = make_args(p, k);
    a.in = p->keep ? p->layers[k - 1] : p->layers[(k - 1) % 2];
    a.out = p->keep ? p->layers[k] : p->layers[k % 2];
    a.ucol = p->ucols_d + (size_t)(k - 1) * m * B;
    a.tail = p->tp_d;
    const bool fuse = probs && k == p->n;
    const int rc = fuse ? dispatch(p->prec, Kern::FwdProb, a, grid_for_units(a, true), s, 0, nullptr, probs)
                        : dispatch(p->prec, Kern::Fwd, a, grid_for_units(a, B == 1), s);
    if (rc != 0) {
      set_error("SLOS layer %d launch failed: %s", k, cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
  }
  p->forwarded = probs == nullptr;
  return PCVL_OK;
}

extern "C" int pcvl_slos_forward(pcvl_slos_plan* p, const double* u_d, void* stream) {
  PCVL_CHECK(p && u_d, "null pointer argument");
  return forward(p, u_d, (size_t)p->m * p->m, (cudaStream_t)stream);
}

extern "C" int pcvl_slos_forward_shared(pcvl_slos_plan* p, const double* u_d, void* stream) {
  PCVL_CHECK(p && u_d, "null pointer argument");
  return forward(p, u_d, 0, (cudaStream_t)stream);
}

static int finalize(pcvl_slos_plan* p, int mode, const double* w, double* out_real, double2* out_c, void* seed,
                    cudaStream_t s);

extern "C" int pcvl_slos_forward_probabilities(pcvl_slos_plan* p, const double* u_d, double* probs_d, void* stream) {
  PCVL_CHECK(p && u_d && probs_d, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t ustride = (size_t)p->m * p->m;
  if (p->masked || p->B > 1 || p->n == 0) {  // forward, then the probabilities of the stored last layer
    PCVL_TRY(forward(p, u_d, ustride, s));
    return finalize(p, 0, nullptr, probs_d, nullptr, nullptr, s);
  }
  return forward(p, u_d, ustride, s, probs_d);
}

static int finalize(pcvl_slos_plan* p, int mode, const double* w, double* out_real, double2* out_c, void* seed,
                    cudaStream_t s) {
  PCVL_CHECK(p->forwarded, "pcvl_slos_forward has not run on this plan");
  if (p->masked) return slos_masked_finalize(p, mode, w, out_real, out_c, seed, s);
  SlosArgs a = make_args(p, p->n);
  a.in = p->final_layer();
  const int rc = dispatch(p->prec, Kern::Fin, a, grid_for_units(a, p->B == 1), s, mode, w, out_real, out_c, seed);
  if (rc != 0) {
    set_error("SLOS finalize launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return PCVL_ERR_CUDA;
  }
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
  PCVL_CHECK(p->forwarded, "pcvl_slos_forward has not run on this plan");
  cudaStream_t s = (cudaStream_t)stream_;
  if (p->masked) return slos_masked_backward(p, weights_d, grad_u_d, s);
  const int m = p->m, B = p->B, n = p->n;
  PCVL_CUDA(cudaMemsetAsync(grad_u_d, 0, (size_t)B * m * m * 2 * sizeof(double), s));
  PCVL_TRY(finalize(p, 2, weights_d, nullptr, nullptr, p->adj_d[n % 2], s));
  for (int k = n; k >= 1; --k) {
    SlosArgs a = make_args(p, k - 1, kChunkBwdB);  // tiles of the parent layer
    a.in = p->adj_d[k % 2];
    a.out = p->adj_d[(k - 1) % 2];
    a.ucol = p->ucols_d + (size_t)(k - 1) * m * B;
    a.cpar = p->layers[k - 1];
    a.gpart = p->gpart_d;
    a.tail = p->tc_d;
    const int grid = std::min(p->gpart_blocks, grid_for_units(a));
    const int rc = dispatch(p->prec, Kern::Bwd, a, grid, s);
    if (rc != 0) {
      set_error("SLOS adjoint layer %d launch failed: %s", k, cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
    if (p->prec == kPrecFP64)
      slos_grad_reduce<Arith64><<<(m * B + 255) / 256, 256, 0, s>>>(
          (const double2*)p->gpart_d, grid, m, B, p->col_d + (size_t)(k - 1) * B, (double2*)grad_u_d);
    else
      slos_grad_reduce<ArithFF><<<(m * B + 255) / 256, 256, 0, s>>>(
          p->gpart_d, grid, m, B, p->col_d + (size_t)(k - 1) * B, (double2*)grad_u_d);
    PCVL_CUDA(cudaGetLastError());
  }
  return PCVL_OK;
}
