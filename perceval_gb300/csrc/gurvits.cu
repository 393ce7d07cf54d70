// Monte-Carlo permanent estimates (Gurvits' randomised estimator) with a 99% bound.
//
// Replaces xq.estimate_permanent_cx(M, iterations) -> (estimate, error), called by
// NaiveApproxBackend (perceval/backends/_naive_approx.py:52-59).  For an n x n complex
// matrix A and x uniform on {-1, +1}^n,
//     X(x) = (prod_i x_i) prod_j (sum_i x_i a_ij)
// has mean Perm(A) (Glynn's formula read as an expectation; Gurvits 2005), and by the
// AM-GM inequality |X(x)| <= (|A^T x|^2 / n)^(n/2) <= ||A||_2^n =: B.  The estimate is
// the mean of N independent draws.  Its bound applies Hoeffding's inequality to the real
// and imaginary parts (each in [-B, B], failure probability 0.005 each):
//     |mean - Perm(A)| <= B sqrt(4 ln(400) / N)   with probability >= 0.99.
// B uses a rigorous upper bound of the spectral norm: for M = A^H A (Hermitian, PSD),
//     lambda_max(M) <= (tr M^(2^q))^(2^-q)
// evaluated in FP64 by q = 12 renormalised squarings; it exceeds ||A||_2 by at most the
// factor n^(2^-(q+1)) (< 1.0005 for n <= 40).
//
// Draw k of matrix i (global index first + i * iterations + k) takes its n <= 40 signs
// from the 128 bits of Philox4x32-10 with key = seed and counter
// (index lo, index hi, 0x67757276, 0): bit r set means x_r = -1.
//
// Kernels: gv_norm (one CTA per matrix: the bound, and a power-of-two scale 2^-e with
// 2^e >= the norm bound, so every draw of the scaled matrix has |X| <= 1 and every
// partial product stays far inside the FP32 range), gv_sample (FP32 column sums and
// products per draw, FP64 accumulation, one partial per CTA), gv_reduce (per matrix:
// compensated sum of the partials, undo the scale, the bound).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "runtime.cuh"

namespace pcvl {

constexpr int kGvMaxN = 40;
constexpr int kGvSquarings = 12;
constexpr int kGvThreads = 256;
constexpr uint32_t kGvTag = 0x67757276u;

struct GvDesc {
  int64_t off;      // first element of the matrix
  int64_t part;     // first partial of the matrix
  int32_t n;
  int32_t chunks;   // CTAs (partials) of the matrix
};

// ---------------------------------------------------------------- norm bound
// Float-float on the FP32 pipe (GB300's FP64 rate would make this the costliest part of a
// call).  The matrix is first scaled by 2^-ea (ea: exponent of its largest entry) so every
// product stays far inside the FP32 range; the bound is unscaled at the end.
// Dynamic shared memory: A (n x n), M and M^2 (n x n each), float-float complex.
__global__ void __launch_bounds__(128) gv_norm(const double2* __restrict__ mats, const GvDesc* __restrict__ descs,
                                               double* __restrict__ log2_bound, int32_t* __restrict__ scale_exp) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GvDesc d = descs[blockIdx.x];
  const int n = d.n, tid = threadIdx.x;
  cdd* A = reinterpret_cast<cdd*>(smem);
  cdd* M = A + n * n;
  cdd* M2 = M + n * n;
  __shared__ double red[128];
  __shared__ double s_log2;  // log2 of the running bound on lambda_max(A^H A), scaled A
  if (n == 0) {
    if (tid == 0) {
      log2_bound[blockIdx.x] = 0.0;
      scale_exp[blockIdx.x] = 0;
    }
    return;
  }
  // largest |entry| -> exponent ea
  double amax = 0.0;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const double2 v = mats[d.off + e];
    amax = fmax(amax, fmax(fabs(v.x), fabs(v.y)));
  }
  red[tid] = amax;
  __syncthreads();
  for (int st = 64; st > 0; st >>= 1) {
    if (tid < st) red[tid] = fmax(red[tid], red[tid + st]);
    __syncthreads();
  }
  const int ea = red[0] > 0.0 ? ilogb(red[0]) + 1 : 0;
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) {
    const double2 v = mats[d.off + e];
    A[e] = cdd_from(ldexp(v.x, -ea), ldexp(v.y, -ea));
  }
  __syncthreads();
  // M = A^H A: M_ij = sum_k conj(a_ki) a_kj
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    cacc acc = cacc_zero();
    for (int k = 0; k < n; ++k) cacc_fma(acc, cdd_conj(A[k * n + i]), A[k * n + j]);
    M[e] = cacc_finish(acc);
  }
  __syncthreads();
  // trace-normalised repeated squaring
  for (int q = 0; q <= kGvSquarings; ++q) {
    double t = 0.0;
    for (int i = tid; i < n; i += blockDim.x) t += dd_to_double(M[i * n + i].re);
    red[tid] = t;
    __syncthreads();
    for (int st = 64; st > 0; st >>= 1) {
      if (tid < st) red[tid] += red[tid + st];
      __syncthreads();
    }
    const double tr = red[0];
    if (tid == 0) {
      // q = 0: lambda_max(M) <= tr M; q >= 1: factor (tr M_q)^(2^-q) with M_q = M_{q-1}^2
      const double w = q == 0 ? 1.0 : ldexp(1.0, -q);
      s_log2 = (q == 0 ? 0.0 : s_log2) + (tr > 0.0 ? w * log2(tr) : -INFINITY);
    }
    __syncthreads();
    if (!(tr > 0.0) || q == kGvSquarings) break;
    const dd inv = dd_from_double(1.0 / tr);
    for (int e = tid; e < n * n; e += blockDim.x) M[e] = {dd_mul(M[e].re, inv), dd_mul(M[e].im, inv)};
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) {
      const int i = e / n, j = e - i * n;
      cacc acc = cacc_zero();
      for (int k = 0; k < n; ++k) cacc_fma(acc, M[i * n + k], M[k * n + j]);
      M2[e] = cacc_finish(acc);
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) M[e] = M2[e];
    __syncthreads();
  }
  if (tid == 0) {
    const double l2 = s_log2;                 // log2 bound of lambda_max = ||A'||_2^2, A' = 2^-ea A
    const double lnorm = 0.5 * l2 + ea;       // log2 bound of ||A||_2
    log2_bound[blockIdx.x] = isfinite(l2) ? n * lnorm : -INFINITY;
    scale_exp[blockIdx.x] = isfinite(l2) ? (int)ceil(lnorm) : 0;
  }
}

// ---------------------------------------------------------------- draws
struct GvArgs {
  const double2* mats;
  const GvDesc* descs;
  const int32_t* scale_exp;
  const int32_t* cta_mat;   // matrix of every CTA
  int64_t iterations;
  uint64_t first;
  uint32_t k0, k1;
  double2* partials;
};

template <int NMAX>
__global__ void __launch_bounds__(kGvThreads) gv_sample(GvArgs a) {
  // rows padded to an even length (a zero column for odd n): two adjacent columns are one
  // 16-byte load, so each load of the matrix feeds four multiply-adds
  constexpr int NS = (NMAX + 1) & ~1;
  __shared__ __align__(16) float2 As[NMAX * NS];
  __shared__ double2 red[kGvThreads / 32];
  const int mi = a.cta_mat[blockIdx.x];
  const GvDesc d = a.descs[mi];
  const int n = d.n, tid = threadIdx.x;
  const int c = (int)((int64_t)blockIdx.x - d.part);  // CTA index = partial index
  const int e = a.scale_exp[mi];
  const int ns = (n + 1) & ~1;
  for (int x = tid; x < n * ns; x += blockDim.x) {
    const int i = x / ns, j = x - i * ns;
    const double2 v = j < n ? a.mats[d.off + (int64_t)i * n + j] : make_double2(0.0, 0.0);
    As[x] = make_float2((float)ldexp(v.x, -e), (float)ldexp(v.y, -e));
  }
  __syncthreads();
  double sr = 0.0, si = 0.0;
  const int64_t per = (a.iterations + d.chunks - 1) / d.chunks;
  const int64_t k_begin = (int64_t)c * per;
  const int64_t k_end = min(a.iterations, k_begin + per);
  const uint64_t base = a.first + (uint64_t)mi * (uint64_t)a.iterations;
  for (int64_t k = k_begin + tid; k < k_end; k += blockDim.x) {
    const uint64_t idx = base + (uint64_t)k;
    const u4 r = philox4x32_10({(uint32_t)idx, (uint32_t)(idx >> 32), kGvTag, 0u}, a.k0, a.k1);
    float s[NMAX];
    int par = 0;
#pragma unroll
    for (int i = 0; i < NMAX; ++i) {
      const uint32_t w = i < 32 ? r.x : r.y;
      const int bit = (int)((w >> (i & 31)) & 1u);
      s[i] = bit ? -1.f : 1.f;
      if (i < n) par ^= bit;
    }
    float pr = 1.f, pi = 0.f;
    for (int j = 0; j < n; j += 2) {
      float yr = 0.f, yi = 0.f, zr = 0.f, zi = 0.f;  // columns j and j + 1
#pragma unroll
      for (int i = 0; i < NMAX; ++i) {
        if (i < n) {
          const float4 v = *reinterpret_cast<const float4*>(&As[i * ns + j]);
          yr = fmaf(s[i], v.x, yr);
          yi = fmaf(s[i], v.y, yi);
          zr = fmaf(s[i], v.z, zr);
          zi = fmaf(s[i], v.w, zi);
        }
      }
      float tr = pr * yr - pi * yi;
      pi = fmaf(pr, yi, pi * yr);
      pr = tr;
      if (j + 1 < n) {
        tr = pr * zr - pi * zi;
        pi = fmaf(pr, zi, pi * zr);
        pr = tr;
      }
    }
    if (par) {
      pr = -pr;
      pi = -pi;
    }
    sr += (double)pr;
    si += (double)pi;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if ((tid & 31) == 0) red[tid >> 5] = make_double2(sr, si);
  __syncthreads();
  if (tid == 0) {
    double2 t = red[0];
    for (int w = 1; w < kGvThreads / 32; ++w) {
      t.x += red[w].x;
      t.y += red[w].y;
    }
    a.partials[blockIdx.x] = t;
  }
}

__global__ void gv_reduce(const double2* __restrict__ mats, const GvDesc* __restrict__ descs,
                          const double2* __restrict__ partials, const double* __restrict__ log2_bound,
                          const int32_t* __restrict__ scale_exp, int32_t count, int64_t iterations,
                          double2* __restrict__ out, double* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const GvDesc d = descs[i];
  if (d.n == 0) {
    out[i] = make_double2(1.0, 0.0);
    err[i] = 0.0;
    return;
  }
  if (d.n == 1) {  // X(x) = x^2 a = a for every draw: exact
    out[i] = mats[d.off];
    err[i] = 0.0;
    return;
  }
  double sr = 0.0, cr = 0.0, si = 0.0, ci = 0.0;
  for (int c = 0; c < d.chunks; ++c) {
    const double2 p = partials[d.part + c];
    double t = sr + p.x;
    cr += fabs(sr) >= fabs(p.x) ? (sr - t) + p.x : (p.x - t) + sr;
    sr = t;
    t = si + p.y;
    ci += fabs(si) >= fabs(p.y) ? (si - t) + p.y : (p.y - t) + si;
    si = t;
  }
  const int sh = d.n * scale_exp[i];
  const double invN = 1.0 / (double)iterations;
  out[i] = make_double2(ldexp((sr + cr) * invN, sh), ldexp((si + ci) * invN, sh));
  const double lb = log2_bound[i];
  err[i] = isfinite(lb) ? exp2(lb) * sqrt(4.0 * log(400.0) * invN) : 0.0;
}

template <int NMAX>
static int launch_gv(const GvArgs& a, int64_t ctas, cudaStream_t s) {
  gv_sample<NMAX><<<(unsigned)ctas, kGvThreads, 0, s>>>(a);
  return (int)cudaGetLastError();
}

}  // namespace pcvl

using namespace pcvl;

extern "C" int pcvl_permanent_estimate_batch(const double* mats_d, const int64_t* offsets_h, const int32_t* sizes_h,
                                             int32_t count, int64_t iterations, uint64_t seed, uint64_t first_sample,
                                             double* out_d, double* err_d, void* stream_) {
  cudaStream_t s = (cudaStream_t)stream_;
  PCVL_CHECK(count >= 0, "count must be >= 0 (got %d)", count);
  if (count == 0) return PCVL_OK;
  PCVL_CHECK(mats_d && offsets_h && sizes_h && out_d && err_d, "null pointer argument");
  PCVL_CHECK(iterations >= 1, "iterations must be >= 1 (got %lld)", (long long)iterations);
  int nmax = 0;
  for (int i = 0; i < count; ++i) {
    PCVL_CHECK(sizes_h[i] >= 0 && sizes_h[i] <= kGvMaxN, "matrix %d: size %d outside [0, %d]", i, sizes_h[i],
               kGvMaxN);
    PCVL_CHECK(offsets_h[i] >= 0, "matrix %d: negative offset", i);
    nmax = std::max(nmax, (int)sizes_h[i]);
  }
  // CTAs per matrix: enough CTAs for the chip, at least 256 draws per CTA
  const int sms = num_sms();
  const int64_t want = std::max<int64_t>(1, (int64_t)8 * sms / count);
  const int64_t cap = std::max<int64_t>(1, iterations / kGvThreads);
  const int chunks = (int)std::min<int64_t>(want, cap);
  std::vector<GvDesc> descs(count);
  std::vector<int32_t> cta_mat;
  int64_t parts = 0;
  for (int i = 0; i < count; ++i) {
    const int n = sizes_h[i];
    const int c = n >= 2 ? chunks : 0;
    descs[i] = {offsets_h[i], parts, n, c};
    for (int k = 0; k < c; ++k) cta_mat.push_back(i);
    parts += c;
  }
  const size_t o_desc = 0;
  const size_t o_cta = align_up(o_desc + (size_t)count * sizeof(GvDesc), 256);
  const size_t o_part = align_up(o_cta + (size_t)std::max<int64_t>(parts, 1) * 4, 256);
  const size_t o_lb = align_up(o_part + (size_t)std::max<int64_t>(parts, 1) * sizeof(double2), 256);
  const size_t o_se = align_up(o_lb + (size_t)count * 8, 256);
  const size_t total = align_up(o_se + (size_t)count * 4, 256);
  std::vector<unsigned char> blob(o_part - o_desc, 0);
  memcpy(blob.data(), descs.data(), (size_t)count * sizeof(GvDesc));
  if (!cta_mat.empty()) memcpy(blob.data() + o_cta, cta_mat.data(), cta_mat.size() * 4);
  ScratchGuard scratch(s);
  void* ws = nullptr;
  PCVL_TRY(scratch.alloc(total, &ws));
  unsigned char* base = (unsigned char*)ws;
  PCVL_TRY(stage_h2d(blob.data(), blob.size(), base, s));
  const GvDesc* descs_d = (const GvDesc*)(base + o_desc);
  double* lb_d = (double*)(base + o_lb);
  int32_t* se_d = (int32_t*)(base + o_se);
  double2* part_d = (double2*)(base + o_part);

  const size_t nsmem = (size_t)3 * nmax * nmax * sizeof(double2);
  if (nsmem > 48 * 1024)
    PCVL_CUDA(cudaFuncSetAttribute(gv_norm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nsmem));
  gv_norm<<<count, 128, nsmem, s>>>((const double2*)mats_d, descs_d, lb_d, se_d);
  PCVL_CUDA(cudaGetLastError());
  if (parts > 0) {
    GvArgs a{};
    a.mats = (const double2*)mats_d;
    a.descs = descs_d;
    a.scale_exp = se_d;
    a.cta_mat = (const int32_t*)(base + o_cta);
    a.iterations = iterations;
    a.first = first_sample;
    a.k0 = (uint32_t)seed;
    a.k1 = (uint32_t)(seed >> 32);
    a.partials = part_d;
    int rc;
    if (nmax <= 8)
      rc = launch_gv<8>(a, parts, s);
    else if (nmax <= 16)
      rc = launch_gv<16>(a, parts, s);
    else if (nmax <= 24)
      rc = launch_gv<24>(a, parts, s);
    else if (nmax <= 32)
      rc = launch_gv<32>(a, parts, s);
    else
      rc = launch_gv<40>(a, parts, s);
    if (rc != 0) {
      set_error("permanent estimate launch failed: %s", cudaGetErrorString((cudaError_t)rc));
      return PCVL_ERR_CUDA;
    }
  }
  gv_reduce<<<(count + 127) / 128, 128, 0, s>>>((const double2*)mats_d, descs_d, part_d, lb_d, se_d, count,
                                                 iterations, (double2*)out_d, err_d);
  PCVL_CUDA(cudaGetLastError());
  return PCVL_OK;
}
