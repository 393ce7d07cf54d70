/*
 * CPU oracle for the linear-optics hot path.  TEST INFRASTRUCTURE ONLY: the
 * library's product path never calls into this file; tests and the smoke check use
 * it to check results, the benchmark to time the CPU baseline.
 *
 * Plain FP64 restatement of the reference semantics (the reference's arithmetic
 * lives in the closed exqalibur~=1.1.0 library; its call sites and tests fix what
 * is computed):
 *  - permanents: perceval/backends/_naive.py:46-71 (xq.permanent_cx), Glynn (2010)
 *    Gray-code formula and Ryser (1963) formula, docs/source/backends.rst:160-167;
 *  - SLOS: perceval/backends/_slos.py:37-223 (path order :61-86, layer update
 *    :93-99, normalisation :187-214);
 *  - Clifford & Clifford (2018) algorithm B: perceval/backends/_clifford2017.py,
 *    docs/source/backends.rst:104-116, with the same Philox4x32-10 stream and
 *    draw procedure as the GPU sampler so samples can be compared one by one;
 *  - Gurvits' randomised permanent estimator (xq.estimate_permanent_cx, called at
 *    perceval/backends/_naive_approx.py:52-59; docs/source/backends.rst:182-187), with
 *    the same sign draws as the GPU estimator.
 * Fock states of n photons on m modes are ranked in descending lexicographic order
 * (tests/utils/test_statevector.py:430-438).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* ---------------------------------------------------------------- combinatorics */
static uint64_t fock_count(int M, int k) {
  if (k < 0) return 0;
  if (M <= 0) return k == 0 ? 1 : 0;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (uint64_t)(M - 1 + i) / (uint64_t)i;
  return r;
}

uint64_t oracle_fock_count(int m, int n) { return fock_count(m, n); }

/* rank in descending-lex order: sum_i Cn(m - i, R_{i+1} - 1) */
uint64_t oracle_fock_rank(int m, const int* s) {
  int rest = 0;
  for (int i = 0; i < m; ++i) rest += s[i];
  uint64_t r = 0;
  for (int i = 0; i < m; ++i) {
    rest -= s[i];
    if (rest > 0) r += fock_count(m - i, rest - 1);
  }
  return r;
}

void oracle_fock_unrank(int m, int n, uint64_t rank, int* s) {
  int rest = n;
  for (int i = 0; i < m - 1; ++i) {
    int v = rest;
    for (;;) {
      uint64_t blk = fock_count(m - i - 1, rest - v);
      if (rank < blk) break;
      rank -= blk;
      --v;
    }
    s[i] = v;
    rest -= v;
  }
  s[m - 1] = rest;
}

/* next state in descending-lex order; returns 0 after the last one */
static int fock_next(int m, int* s) {
  int tail = 0;
  for (int i = m - 2; i >= 0; --i) {
    tail += s[i + 1];
    if (s[i] > 0) {
      s[i] -= 1;
      s[i + 1] = tail + 1;
      for (int j = i + 2; j < m; ++j) s[j] = 0;
      return 1;
    }
  }
  return 0;
}

/* ---------------------------------------------------------------- permanents */
static void neumaier(double* s, double* c, double x) {
  double t = *s + x;
  if (fabs(*s) >= fabs(x))
    *c += (*s - t) + x;
  else
    *c += (x - t) + *s;
  *s = t;
}

/* Glynn with Gray-code order, restarted from exact row sums every 2^12 steps;
 * a: n x n complex128 row-major (interleaved re, im); out: 2 doubles */
void oracle_perm_glynn(int n, const double* a_, double* out) {
  const cplx* a = (const cplx*)a_;
  if (n == 0) {
    out[0] = 1;
    out[1] = 0;
    return;
  }
  const uint64_t total = 1ull << (n - 1);
  const uint64_t chunk = 1ull << 12;
  const int64_t nchunks = (int64_t)((total + chunk - 1) / chunk);
  double sr = 0, cr = 0, si = 0, ci = 0;
#pragma omp parallel
  {
    double lsr = 0, lcr = 0, lsi = 0, lci = 0;
    cplx* r = (cplx*)malloc(sizeof(cplx) * n);
#pragma omp for schedule(dynamic, 1)
    for (int64_t q = 0; q < nchunks; ++q) {
      const uint64_t g0 = (uint64_t)q * chunk;
      const uint64_t g1 = g0 + chunk < total ? g0 + chunk : total;
      /* delta for Gray code g(k) = k ^ (k >> 1): bit t set -> column t + 1 negative */
      uint64_t gc = g0 ^ (g0 >> 1);
      for (int i = 0; i < n; ++i) {
        cplx v = a[i * n];
        for (int j = 1; j < n; ++j) v += ((gc >> (j - 1)) & 1) ? -a[i * n + j] : a[i * n + j];
        r[i] = v;
      }
      int sign = __builtin_popcountll(gc) & 1;
      for (uint64_t k = g0; k < g1; ++k) {
        if (k > g0) {
          const int t = __builtin_ctzll(k);
          const int j = t + 1;
          gc ^= 1ull << t;
          const int neg = (gc >> t) & 1;
          for (int i = 0; i < n; ++i) r[i] += neg ? -2.0 * a[i * n + j] : 2.0 * a[i * n + j];
          sign ^= 1;
        }
        cplx p = r[0];
        for (int i = 1; i < n; ++i) p *= r[i];
        if (sign) p = -p;
        neumaier(&lsr, &lcr, creal(p));
        neumaier(&lsi, &lci, cimag(p));
      }
    }
    free(r);
#pragma omp critical
    {
      neumaier(&sr, &cr, lsr);
      neumaier(&sr, &cr, lcr);
      neumaier(&si, &ci, lsi);
      neumaier(&si, &ci, lci);
    }
  }
  out[0] = ldexp(sr + cr, -(n - 1));
  out[1] = ldexp(si + ci, -(n - 1));
}

/* Ryser: (-1)^n sum_S (-1)^|S| prod_i sum_{j in S} a_ij, Gray-code over subsets */
void oracle_perm_ryser(int n, const double* a_, double* out) {
  const cplx* a = (const cplx*)a_;
  if (n == 0) {
    out[0] = 1;
    out[1] = 0;
    return;
  }
  const uint64_t total = 1ull << n;
  const uint64_t chunk = 1ull << 12;
  const int64_t nchunks = (int64_t)((total + chunk - 1) / chunk);
  double sr = 0, cr = 0, si = 0, ci = 0;
#pragma omp parallel
  {
    double lsr = 0, lcr = 0, lsi = 0, lci = 0;
    cplx* r = (cplx*)malloc(sizeof(cplx) * n);
#pragma omp for schedule(dynamic, 1)
    for (int64_t q = 0; q < nchunks; ++q) {
      const uint64_t g0 = (uint64_t)q * chunk;
      const uint64_t g1 = g0 + chunk < total ? g0 + chunk : total;
      uint64_t gc = g0 ^ (g0 >> 1);
      for (int i = 0; i < n; ++i) {
        cplx v = 0;
        for (int j = 0; j < n; ++j)
          if ((gc >> j) & 1) v += a[i * n + j];
        r[i] = v;
      }
      for (uint64_t k = g0; k < g1; ++k) {
        if (k > g0) {
          const int t = __builtin_ctzll(k);
          gc ^= 1ull << t;
          const int in = (gc >> t) & 1;
          for (int i = 0; i < n; ++i) r[i] += in ? a[i * n + t] : -a[i * n + t];
        }
        cplx p = r[0];
        for (int i = 1; i < n; ++i) p *= r[i];
        if (__builtin_popcountll(gc) & 1) p = -p;
        neumaier(&lsr, &lcr, creal(p));
        neumaier(&lsi, &lci, cimag(p));
      }
    }
    free(r);
#pragma omp critical
    {
      neumaier(&sr, &cr, lsr);
      neumaier(&sr, &cr, lcr);
      neumaier(&si, &ci, lsi);
      neumaier(&si, &ci, lci);
    }
  }
  const double sg = (n & 1) ? -1.0 : 1.0;
  out[0] = sg * (sr + cr);
  out[1] = sg * (si + ci);
}

/* batch of permanents (packed like the GPU entry point) */
void oracle_perm_batch(const double* mats, const int64_t* offs, const int32_t* sizes, int count, int ryser,
                       double* out) {
  for (int i = 0; i < count; ++i) {
    if (ryser)
      oracle_perm_ryser(sizes[i], mats + 2 * offs[i], out + 2 * i);
    else
      oracle_perm_glynn(sizes[i], mats + 2 * offs[i], out + 2 * i);
  }
}

/* ---------------------------------------------------------------- SLOS */
/* photon order of _Path._decompose for a single input state (_slos.py:61-86) */
int oracle_slos_order(int m, const int* in, int* order) {
  int* c = (int*)malloc(sizeof(int) * m);
  memcpy(c, in, sizeof(int) * m);
  int k = 0;
  for (;;) {
    int best = -1, bv = 0;
    for (int i = 0; i < m; ++i)
      if (c[i] > bv) {
        bv = c[i];
        best = i;
      }
    if (best < 0) break;
    order[k++] = best;
    c[best]--;
  }
  free(c);
  return k;
}

/* one layer: child coefficient = sum_j U[j, mk] * parent(child - e_j), children in
 * rank order, parallel over children */
static void slos_layer(int m, int k, const cplx* U, int mk, const cplx* prev, cplx* cur) {
  const int64_t nc = (int64_t)fock_count(m, k);
#pragma omp parallel
  {
    int* s = (int*)malloc(sizeof(int) * m);
#pragma omp for schedule(static, 4096)
    for (int64_t c = 0; c < nc; ++c) {
      oracle_fock_unrank(m, k, (uint64_t)c, s);
      cplx acc = 0;
      for (int j = 0; j < m; ++j) {
        if (s[j] == 0) continue;
        s[j]--;
        acc += U[j * m + mk] * prev[oracle_fock_rank(m, s)];
        s[j]++;
      }
      cur[c] = acc;
    }
    free(s);
  }
}

/* Final-layer coefficients c_n (rank order) of input `in` through U (m x m). */
int oracle_slos_coefs(int m, const int* in, const double* U_, double* coefs_out) {
  const cplx* U = (const cplx*)U_;
  int n = 0;
  for (int i = 0; i < m; ++i) n += in[i];
  int* order = (int*)malloc(sizeof(int) * (n + 1));
  oracle_slos_order(m, in, order);
  uint64_t mx = 1;
  for (int k = 0; k <= n; ++k)
    if (fock_count(m, k) > mx) mx = fock_count(m, k);
  cplx* a = (cplx*)malloc(sizeof(cplx) * mx);
  cplx* b = (cplx*)malloc(sizeof(cplx) * mx);
  if (!a || !b) {
    free(a);
    free(b);
    free(order);
    return 1;
  }
  a[0] = 1;
  for (int k = 1; k <= n; ++k) {
    slos_layer(m, k, U, order[k - 1], a, b);
    cplx* t = a;
    a = b;
    b = t;
  }
  memcpy(coefs_out, a, sizeof(cplx) * fock_count(m, n));
  free(a);
  free(b);
  free(order);
  return 0;
}

static double prodfact(int m, const int* s) {
  double p = 1;
  for (int i = 0; i < m; ++i)
    for (int v = 2; v <= s[i]; ++v) p *= v;
  return p;
}

/* probabilities |c|^2 prod(out!) / prod(in!) and amplitudes c sqrt(prod(out!)/prod(in!)) */
int oracle_slos(int m, const int* in, const double* U, double* probs, double* amps) {
  int n = 0;
  for (int i = 0; i < m; ++i) n += in[i];
  const int64_t N = (int64_t)fock_count(m, n);
  double* c = (double*)malloc(sizeof(double) * 2 * N);
  if (!c) return 1;
  if (oracle_slos_coefs(m, in, U, c)) {
    free(c);
    return 1;
  }
  const double pin = prodfact(m, in);
  int* s = (int*)calloc(m, sizeof(int));
  s[0] = n;
  for (int64_t r = 0; r < N; ++r) {
    const double f = prodfact(m, s) / pin;
    const double re = c[2 * r], im = c[2 * r + 1];
    if (probs) probs[r] = (re * re + im * im) * f;
    if (amps) {
      amps[2 * r] = re * sqrt(f);
      amps[2 * r + 1] = im * sqrt(f);
    }
    if (!fock_next(m, s)) break;
  }
  free(s);
  free(c);
  return 0;
}

/* dL/dU (torch convention dL/dRe + i dL/dIm) of L = sum_r w[r] p[r] by a reverse
 * sweep over stored layers */
int oracle_slos_grad(int m, const int* in, const double* U_, const double* w, double* grad_) {
  const cplx* U = (const cplx*)U_;
  cplx* grad = (cplx*)grad_;
  int n = 0;
  for (int i = 0; i < m; ++i) n += in[i];
  int* order = (int*)malloc(sizeof(int) * (n + 1));
  oracle_slos_order(m, in, order);
  cplx** L = (cplx**)malloc(sizeof(cplx*) * (n + 1));
  L[0] = (cplx*)malloc(sizeof(cplx));
  L[0][0] = 1;
  for (int k = 1; k <= n; ++k) L[k] = (cplx*)malloc(sizeof(cplx) * fock_count(m, k));
  for (int k = 1; k <= n; ++k) slos_layer(m, k, U, order[k - 1], L[k - 1], L[k]);
  for (int i = 0; i < m * m; ++i) grad[i] = 0;
  const double pin = prodfact(m, in);
  const int64_t N = (int64_t)fock_count(m, n);
  cplx* adj = (cplx*)malloc(sizeof(cplx) * N);
  int* s = (int*)calloc(m, sizeof(int));
  s[0] = n;
  for (int64_t r = 0; r < N; ++r) {
    adj[r] = 2.0 * w[r] * (prodfact(m, s) / pin) * L[n][r];
    if (!fock_next(m, s)) break;
  }
  for (int k = n; k >= 1; --k) {
    const int mk = order[k - 1];
    const int64_t np = (int64_t)fock_count(m, k - 1);
    cplx* pa = (cplx*)malloc(sizeof(cplx) * (np > 0 ? np : 1));
    for (int64_t p = 0; p < np; ++p) {
      oracle_fock_unrank(m, k - 1, (uint64_t)p, s);
      cplx acc = 0;
      for (int j = 0; j < m; ++j) {
        s[j]++;
        const cplx x = adj[oracle_fock_rank(m, s)];
        s[j]--;
        acc += conj(U[j * m + mk]) * x;
        grad[j * m + mk] += conj(L[k - 1][p]) * x;
      }
      pa[p] = acc;
    }
    free(adj);
    adj = pa;
  }
  free(adj);
  free(s);
  for (int k = 0; k <= n; ++k) free(L[k]);
  free(L);
  free(order);
  return 0;
}

/* ---------------------------------------------------------------- Philox4x32-10 */
typedef struct {
  uint32_t x, y, z, w;
} u4;

static u4 philox(u4 c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    u4 d = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    c = d;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

void oracle_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t* out) {
  u4 r = philox((u4){c0, c1, c2, c3}, k0, k1);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

/* permanent of the (rows x cols) selection of U, by Glynn */
static cplx sub_perm(int d, const cplx* U, int m, const int* rows, const int* cols) {
  if (d == 0) return 1;
  double* a = (double*)malloc(sizeof(double) * 2 * d * d);
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      const cplx v = U[rows[r] * m + cols[c]];
      a[2 * (r * d + c)] = creal(v);
      a[2 * (r * d + c) + 1] = cimag(v);
    }
  double o[2];
  oracle_perm_glynn(d, a, o);
  free(a);
  return o[0] + I * o[1];
}

/* Clifford & Clifford algorithm B; out: count x m counts */
void oracle_cc2017(const double* U_, int m, const int* in, int64_t count, uint64_t seed, uint64_t first, int32_t* out) {
  const cplx* U = (const cplx*)U_;
  int n = 0;
  for (int i = 0; i < m; ++i) n += in[i];
  int* cols0 = (int*)malloc(sizeof(int) * (n + 1));
  for (int i = 0, q = 0; i < m; ++i)
    for (int v = 0; v < in[i]; ++v) cols0[q++] = i;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int64_t s = 0; s < count; ++s) {
    const uint64_t sid = first + (uint64_t)s;
    const uint32_t slo = (uint32_t)sid, shi = (uint32_t)(sid >> 32);
    int cols[64], rows[64], subc[64];
    for (int l = 0; l < n; ++l) cols[l] = cols0[l];
    for (int q = n - 1; q >= 1; --q) {
      const u4 r = philox((u4){slo, shi, 0xffffffffu, (uint32_t)q}, k0, k1);
      const int j = (int)(((uint64_t)r.x * (uint64_t)(q + 1)) >> 32);
      const int t = cols[q];
      cols[q] = cols[j];
      cols[j] = t;
    }
    double* w = (double*)malloc(sizeof(double) * m);
    cplx sub[64];
    for (int k = 1; k <= n; ++k) {
      for (int l = 0; l < k; ++l) {
        int q = 0;
        for (int c = 0; c < k; ++c)
          if (c != l) subc[q++] = cols[c];
        sub[l] = sub_perm(k - 1, U, m, rows, subc);
      }
      double W = 0;
      for (int i = 0; i < m; ++i) {
        cplx z = 0;
        for (int l = 0; l < k; ++l) z += U[i * m + cols[l]] * sub[l];
        w[i] = creal(z) * creal(z) + cimag(z) * cimag(z);
        W += w[i];
      }
      const u4 r = philox((u4){slo, shi, (uint32_t)k, 0u}, k0, k1);
      const uint64_t v = ((uint64_t)(r.x >> 5) << 26) | (uint64_t)(r.y >> 6);
      const double target = (double)v * (1.0 / 9007199254740992.0) * W;
      double run = 0;
      int pick = -1, last_pos = 0;
      for (int i = 0; i < m; ++i) {
        if (w[i] > 0) last_pos = i;
        run += w[i];
        if (run > target) {
          pick = i;
          break;
        }
      }
      rows[k - 1] = pick >= 0 ? pick : last_pos;
    }
    free(w);
    int32_t* o = out + s * m;
    for (int i = 0; i < m; ++i) o[i] = 0;
    for (int k = 0; k < n; ++k) o[rows[k]]++;
  }
  free(cols0);
}

/* ---------------------------------------------------------------- Gurvits estimator */
/* One draw: X(x) = (prod_i x_i) prod_j (sum_i x_i a_ij), x_i = -1 where bit i of the
 * 128-bit word w is set (w[0] bits 0..31, w[1] bits 32..63). */
void oracle_glynn_term(int n, const double* a_, const uint32_t* w, double* out) {
  const cplx* a = (const cplx*)a_;
  int par = 0;
  cplx prod = 1;
  for (int i = 0; i < n; ++i) par ^= (int)((w[i >> 5] >> (i & 31)) & 1u);
  for (int j = 0; j < n; ++j) {
    cplx y = 0;
    for (int i = 0; i < n; ++i) {
      const double sgn = ((w[i >> 5] >> (i & 31)) & 1u) ? -1.0 : 1.0;
      y += sgn * a[i * n + j];
    }
    prod *= y;
  }
  if (par) prod = -prod;
  out[0] = creal(prod);
  out[1] = cimag(prod);
}

/* Mean of `iterations` draws; draw k has global index first + k and takes its signs
 * from Philox4x32-10 with key = seed and counter (index lo, index hi, 0x67757276, 0). */
void oracle_gurvits(int n, const double* a, int64_t iterations, uint64_t seed, uint64_t first, double* out) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  double sr = 0, cr = 0, si = 0, ci = 0;
  for (int64_t k = 0; k < iterations; ++k) {
    const uint64_t idx = first + (uint64_t)k;
    const u4 r = philox((u4){(uint32_t)idx, (uint32_t)(idx >> 32), 0x67757276u, 0u}, k0, k1);
    const uint32_t w[2] = {r.x, r.y};
    double x[2];
    oracle_glynn_term(n, a, w, x);
    neumaier(&sr, &cr, x[0]);
    neumaier(&si, &ci, x[1]);
  }
  out[0] = (sr + cr) / (double)iterations;
  out[1] = (si + ci) / (double)iterations;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

/* ---------------------------------------------------------------- CPU baseline paths
 * The same formulas, arranged to run fast on the host (this is what the benchmark's CPU
 * baseline times; the functions above stay the plain restatement the tests pin).
 *
 * Batched Glynn: the sign vectors of every matrix are cut into chunks of 2^12 consecutive
 * Gray-code steps; one OpenMP task per (matrix, chunk), so small matrices use every core
 * too.  For n >= 5 a chunk runs sixteen consecutive steps at once in vector lanes
 * (glynn_chunk16); for n <= 4 one step at a time (glynn_chunk: the row sums as separate
 * real and imaginary arrays, the update of a step one vectorisable loop, the product in
 * four independent chains).  A chunk's terms are summed plainly; the chunks of a matrix
 * are added in order with Neumaier compensation, so results do not depend on the thread
 * count.  FP64 throughout. */
/* Multiply-adds may fuse (FMA) here: this is the timed baseline, not the pinned restatement. */
__attribute__((optimize("fp-contract=fast")))
static void glynn_chunk(int n, const double* ar, const double* ai, uint64_t g0, uint64_t g1, double* rr, double* ri,
                        double* out) {
  /* ar, ai: column-major 2 a (ar[j * n + i] = 2 Re a_ij); row sums at Gray code g0 */
  uint64_t gc = g0 ^ (g0 >> 1);
  for (int i = 0; i < n; ++i) {
    double vr = 0.5 * ar[i], vi = 0.5 * ai[i];
    for (int j = 1; j < n; ++j) {
      const double s = ((gc >> (j - 1)) & 1) ? -0.5 : 0.5;
      vr += s * ar[j * n + i];
      vi += s * ai[j * n + i];
    }
    rr[i] = vr;
    ri[i] = vi;
  }
  int sign = __builtin_popcountll(gc) & 1;
  double sr = 0, si = 0;
  for (uint64_t k = g0; k < g1; ++k) {
    if (k > g0) {
      const int t = __builtin_ctzll(k);
      gc ^= 1ull << t;
      const double c = ((gc >> t) & 1) ? -1.0 : 1.0;
      const double* xr = ar + (size_t)(t + 1) * n;
      const double* xi = ai + (size_t)(t + 1) * n;
      for (int i = 0; i < n; ++i) {
        rr[i] += c * xr[i];
        ri[i] += c * xi[i];
      }
      sign ^= 1;
    }
    double pr[4] = {1, 1, 1, 1}, pi[4] = {0, 0, 0, 0};
    int i = 0;
    for (; i + 4 <= n; i += 4)
      for (int q = 0; q < 4; ++q) {
        const double x = pr[q], y = pi[q], u = rr[i + q], v = ri[i + q];
        pr[q] = x * u - y * v;
        pi[q] = x * v + y * u;
      }
    for (; i < n; ++i) {
      const double x = pr[0], y = pi[0], u = rr[i], v = ri[i];
      pr[0] = x * u - y * v;
      pi[0] = x * v + y * u;
    }
    const double ar01 = pr[0] * pr[1] - pi[0] * pi[1], ai01 = pr[0] * pi[1] + pi[0] * pr[1];
    const double ar23 = pr[2] * pr[3] - pi[2] * pi[3], ai23 = pr[2] * pi[3] + pi[2] * pr[3];
    const double p_r = ar01 * ar23 - ai01 * ai23, p_i = ar01 * ai23 + ai01 * ar23;
    if (sign) {
      sr -= p_r;
      si -= p_i;
    } else {
      sr += p_r;
      si += p_i;
    }
  }
  out[0] = sr;
  out[1] = si;
}

/* Sixteen consecutive Gray-code steps k..k+15 (k a multiple of 16) at once, as eight
 * two-lane vectors per row (GCC's generic vectors; one 128-bit operation each on NEON and
 * SSE2).  The lanes start as the row sums of the sixteen steps, walked from k.  The Gray code
 * is reflected: the next block's steps are this block's in reverse order with one more
 * column flipped, t = ctz(k + 16) >= 4, so the lanes stay in place, each block adds
 * +-x_{t+1} to all of them, and the lane order, hence the lanes' sign-vector parities, alternates
 * from block to block (the parity of gray(j) is that of j: +, - within each vector in step
 * order).  Per row and block: one column update and one complex multiply per lane, sixteen
 * independent product chains. */
typedef double v2d __attribute__((vector_size(16)));
enum { kGlynnVecs = 8, kGlynnLanes = 2 * kGlynnVecs };

__attribute__((optimize("fp-contract=fast")))
static void glynn_chunk16(int n, const double* ar, const double* ai, uint64_t g0, uint64_t g1, v2d* lr, v2d* li,
                          double* out) {
  const uint64_t gc0 = g0 ^ (g0 >> 1);
  for (int i = 0; i < n; ++i) {
    double vr = 0.5 * ar[i], vi = 0.5 * ai[i];
    for (int j = 1; j < n; ++j) {
      const double s = ((gc0 >> (j - 1)) & 1) ? -0.5 : 0.5;
      vr += s * ar[j * n + i];
      vi += s * ai[j * n + i];
    }
    double er[kGlynnLanes], ei[kGlynnLanes];
    uint64_t gc = gc0;
    er[0] = vr;
    ei[0] = vi;
    for (int l = 1; l < kGlynnLanes; ++l) {
      const int t = __builtin_ctzll(g0 + l);
      gc ^= 1ull << t;
      const double c = ((gc >> t) & 1) ? -1.0 : 1.0;
      vr += c * ar[(t + 1) * n + i];
      vi += c * ai[(t + 1) * n + i];
      er[l] = vr;
      ei[l] = vi;
    }
    for (int q = 0; q < kGlynnVecs; ++q) {
      lr[kGlynnVecs * i + q] = (v2d){er[2 * q], er[2 * q + 1]};
      li[kGlynnVecs * i + q] = (v2d){ei[2 * q], ei[2 * q + 1]};
    }
  }
  const v2d one = {1, 1}, zero = {0, 0};
  v2d ls = {1, -1}, sr = zero, si = zero;
  for (uint64_t k = g0; k < g1; k += kGlynnLanes) {
    double cn = 0;
    const double *xr = ar + n, *xi = ai + n;
    if (k > g0) {
      const int t = __builtin_ctzll(k);
      cn = (((k ^ (k >> 1)) >> t) & 1) ? -1.0 : 1.0;
      xr = ar + (size_t)(t + 1) * n;
      xi = ai + (size_t)(t + 1) * n;
      ls = -ls;
    }
    v2d pr[kGlynnVecs], pi[kGlynnVecs];
    for (int q = 0; q < kGlynnVecs; ++q) {
      pr[q] = one;
      pi[q] = zero;
    }
    for (int i = 0; i < n; ++i) {
      const double dr = cn * xr[i], di = cn * xi[i];
      for (int q = 0; q < kGlynnVecs; ++q) {
        const v2d u = lr[kGlynnVecs * i + q] + dr, v = li[kGlynnVecs * i + q] + di;
        lr[kGlynnVecs * i + q] = u;
        li[kGlynnVecs * i + q] = v;
        const v2d x = pr[q];
        pr[q] = x * u - pi[q] * v;
        pi[q] = x * v + pi[q] * u;
      }
    }
    for (int q = 0; q < kGlynnVecs; ++q) {
      sr += ls * pr[q];
      si += ls * pi[q];
    }
  }
  out[0] = sr[0] + sr[1];
  out[1] = si[0] + si[1];
}

void oracle_perm_batch_fast(const double* mats, const int64_t* offs, const int32_t* sizes, int count, double* out) {
  const uint64_t chunk = 1ull << 12;
  int64_t* first = (int64_t*)malloc(sizeof(int64_t) * (count + 1));
  first[0] = 0;
  for (int i = 0; i < count; ++i) {
    const int n = sizes[i];
    const uint64_t total = n > 0 ? 1ull << (n - 1) : 0;
    first[i + 1] = first[i] + (int64_t)((total + chunk - 1) / chunk);
  }
  const int64_t ntasks = first[count];
  double* part = (double*)malloc(sizeof(double) * 2 * (ntasks > 0 ? ntasks : 1));
#pragma omp parallel
  {
    double* buf = (double*)malloc(sizeof(double) * (4 * 40 + 4 * 40 * 40));
    v2d* lanes = (v2d*)aligned_alloc(16, sizeof(v2d) * 2 * kGlynnVecs * 40);
    int cur = -1;
    double *ar = buf + 160, *ai = ar + 1600, *rr = buf, *ri = buf + 40;
#pragma omp for schedule(dynamic, 1)
    for (int64_t q = 0; q < ntasks; ++q) {
      int lo = 0, hi = count;  /* matrix of task q: first[mat] <= q < first[mat + 1] */
      while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (first[mid] <= q) lo = mid; else hi = mid;
      }
      while (first[lo + 1] <= q) ++lo;
      const int mat = lo, n = sizes[mat];
      if (mat != cur) {
        const double* a = mats + 2 * offs[mat];
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            ar[j * n + i] = 2.0 * a[2 * (i * n + j)];
            ai[j * n + i] = 2.0 * a[2 * (i * n + j) + 1];
          }
        cur = mat;
      }
      const uint64_t total = 1ull << (n - 1);
      const uint64_t g0 = (uint64_t)(q - first[mat]) * chunk;
      const uint64_t g1 = g0 + chunk < total ? g0 + chunk : total;
      if (n >= 5)  /* chunks of 2^12 steps or of the whole 2^(n-1): multiples of 16 */
        glynn_chunk16(n, ar, ai, g0, g1, lanes, lanes + kGlynnVecs * 40, part + 2 * q);
      else
        glynn_chunk(n, ar, ai, g0, g1, rr, ri, part + 2 * q);
    }
    free(buf);
    free(lanes);
  }
  for (int i = 0; i < count; ++i) {
    const int n = sizes[i];
    if (n == 0) {
      out[2 * i] = 1;
      out[2 * i + 1] = 0;
      continue;
    }
    double sr = 0, cr = 0, si = 0, ci = 0;
    for (int64_t q = first[i]; q < first[i + 1]; ++q) {
      neumaier(&sr, &cr, part[2 * q]);
      neumaier(&si, &ci, part[2 * q + 1]);
    }
    out[2 * i] = ldexp(sr + cr, -(n - 1));
    out[2 * i + 1] = ldexp(si + ci, -(n - 1));
  }
  free(part);
  free(first);
}

/* Clifford & Clifford algorithm B, samples in parallel (the same Philox stream and draw
 * procedure as oracle_cc2017), with the k sub-permanents of a step from one Glynn sum over
 * the signs of the k - 1 chosen rows: for each sign vector d the k column sums
 * c_j = sum_i d_i U[row_i, col_j], and the sub-permanent without column l is
 * 2^(2-k) sum_d (prod d) prod_{j != l} c_j, the leave-one-out products taken from prefix
 * and suffix products.  O(k 2^(k-2)) per step instead of O(k^2 2^(k-2)). */
static void sub_perms_all(int k, const cplx* U, int m, const int* rows, const int* cols, cplx* sub) {
  if (k == 1) {
    sub[0] = 1;
    return;
  }
  const int d = k - 1;  /* rows; sign of row 0 fixed to +1 */
  cplx c[64], pre[65], suf[65];
  double accr[64], acci[64];
  for (int l = 0; l < k; ++l) accr[l] = acci[l] = 0;
  const uint64_t total = 1ull << (d - 1);
  uint64_t gc = 0;
  for (int j = 0; j < k; ++j) {
    cplx v = 0;
    for (int i = 0; i < d; ++i) v += U[rows[i] * m + cols[j]];
    c[j] = v;
  }
  int sign = 0;
  for (uint64_t t = 0; t < total; ++t) {
    if (t > 0) {
      const int b = __builtin_ctzll(t);
      gc ^= 1ull << b;
      const int neg = (gc >> b) & 1;  /* row b + 1 flips */
      for (int j = 0; j < k; ++j) {
        const cplx x = 2.0 * U[rows[b + 1] * m + cols[j]];
        c[j] += neg ? -x : x;
      }
      sign ^= 1;
    }
    pre[0] = 1;
    for (int j = 0; j < k; ++j) pre[j + 1] = pre[j] * c[j];
    suf[k] = 1;
    for (int j = k - 1; j >= 0; --j) suf[j] = suf[j + 1] * c[j];
    for (int l = 0; l < k; ++l) {
      const cplx p = pre[l] * suf[l + 1];
      if (sign) {
        accr[l] -= creal(p);
        acci[l] -= cimag(p);
      } else {
        accr[l] += creal(p);
        acci[l] += cimag(p);
      }
    }
  }
  for (int l = 0; l < k; ++l) sub[l] = ldexp(accr[l], -(d - 1)) + I * ldexp(acci[l], -(d - 1));
}

/* The same sum with 2 kSubVecs consecutive Gray-code steps in vector lanes (kSubVecs two-lane
 * vectors per column; as glynn_chunk16 does for permanents): the lanes start as the column
 * sums of steps 0, 1, ..., walked from t = 0; each later block adds +-x_{b+1}, b = ctz(t)
 * (x_i = 2 U[row_i, cols]), to every lane and reverses the lanes' step order, hence their
 * parity pattern.  Per block the prefix and suffix products run as 2 kSubVecs independent
 * chains.  For k >= kSubMinK (at least one block of steps). */
enum { kSubVecs = 8, kSubLanes = 2 * kSubVecs, kSubMinK = 6 };  /* 2^(kSubMinK - 2) = kSubLanes */

__attribute__((optimize("fp-contract=fast")))
static void sub_perms_lanes(int k, const cplx* U, int m, const int* rows, const int* cols, cplx* sub) {
  const int d = k - 1, V = kSubVecs;
  double ur[d * k], ui[d * k];  /* 2 U[rows[i], cols[j]] */
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < k; ++j) {
      const cplx z = U[rows[i] * m + cols[j]];
      ur[i * k + j] = 2.0 * creal(z);
      ui[i * k + j] = 2.0 * cimag(z);
    }
  v2d cr[k * V], ci[k * V], pr[(k + 1) * V], pi[(k + 1) * V], ar[k * V], ai[k * V];
  const v2d one = {1, 1}, zero = {0, 0};
  for (int j = 0; j < k; ++j) {
    double er[kSubLanes], ei[kSubLanes];
    double vr = 0, vi = 0;
    for (int i = 0; i < d; ++i) {
      vr += 0.5 * ur[i * k + j];
      vi += 0.5 * ui[i * k + j];
    }
    uint64_t gc = 0;
    er[0] = vr;
    ei[0] = vi;
    for (int l = 1; l < kSubLanes; ++l) {
      const int b = __builtin_ctzll((uint64_t)l);
      gc ^= 1ull << b;
      const double c = ((gc >> b) & 1) ? -1.0 : 1.0;
      vr += c * ur[(b + 1) * k + j];
      vi += c * ui[(b + 1) * k + j];
      er[l] = vr;
      ei[l] = vi;
    }
    for (int q = 0; q < V; ++q) {
      cr[j * V + q] = (v2d){er[2 * q], er[2 * q + 1]};
      ci[j * V + q] = (v2d){ei[2 * q], ei[2 * q + 1]};
      ar[j * V + q] = ai[j * V + q] = zero;
    }
  }
  v2d ls = {1, -1};
  const uint64_t total = 1ull << (d - 1);
  for (uint64_t t = 0; t < total; t += kSubLanes) {
    if (t > 0) {
      const int b = __builtin_ctzll(t);
      const double c = (((t ^ (t >> 1)) >> b) & 1) ? -1.0 : 1.0;
      const double *xr = ur + (size_t)(b + 1) * k, *xi = ui + (size_t)(b + 1) * k;
      for (int j = 0; j < k; ++j) {
        const double dr = c * xr[j], di = c * xi[j];
        for (int q = 0; q < V; ++q) {
          cr[j * V + q] += dr;
          ci[j * V + q] += di;
        }
      }
      ls = -ls;
    }
    v2d Pr[kSubVecs], Pi[kSubVecs], Sr[kSubVecs], Si[kSubVecs];
    for (int q = 0; q < V; ++q) {
      Pr[q] = Sr[q] = pr[q] = one;
      Pi[q] = Si[q] = pi[q] = zero;
    }
    for (int j = 0; j < k; ++j)  /* prefix products */
      for (int q = 0; q < V; ++q) {
        const v2d x = Pr[q], u = cr[j * V + q], v = ci[j * V + q];
        Pr[q] = x * u - Pi[q] * v;
        Pi[q] = x * v + Pi[q] * u;
        pr[(j + 1) * V + q] = Pr[q];
        pi[(j + 1) * V + q] = Pi[q];
      }
    for (int j = k - 1; j >= 0; --j)  /* suffix products, and prefix x suffix into the sums */
      for (int q = 0; q < V; ++q) {
        const v2d a = pr[j * V + q], b = pi[j * V + q];
        ar[j * V + q] += ls * (a * Sr[q] - b * Si[q]);
        ai[j * V + q] += ls * (a * Si[q] + b * Sr[q]);
        const v2d x = Sr[q], u = cr[j * V + q], v = ci[j * V + q];
        Sr[q] = x * u - Si[q] * v;
        Si[q] = x * v + Si[q] * u;
      }
  }
  for (int l = 0; l < k; ++l) {
    v2d tr = zero, ti = zero;
    for (int q = 0; q < V; ++q) {
      tr += ar[l * V + q];
      ti += ai[l * V + q];
    }
    sub[l] = ldexp(tr[0] + tr[1], -(d - 1)) + I * ldexp(ti[0] + ti[1], -(d - 1));
  }
}

void oracle_cc2017_fast(const double* U_, int m, const int* in, int64_t count, uint64_t seed, uint64_t first,
                        int32_t* out) {
  const cplx* U = (const cplx*)U_;
  int n = 0;
  for (int i = 0; i < m; ++i) n += in[i];
  int cols0[64];
  for (int i = 0, q = 0; i < m; ++i)
    for (int v = 0; v < in[i]; ++v) cols0[q++] = i;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma omp parallel
  {
    double* w = (double*)malloc(sizeof(double) * m);
#pragma omp for schedule(dynamic, 1)
    for (int64_t s = 0; s < count; ++s) {
      const uint64_t sid = first + (uint64_t)s;
      const uint32_t slo = (uint32_t)sid, shi = (uint32_t)(sid >> 32);
      int cols[64], rows[64];
      cplx sub[64];
      for (int l = 0; l < n; ++l) cols[l] = cols0[l];
      for (int q = n - 1; q >= 1; --q) {
        const u4 r = philox((u4){slo, shi, 0xffffffffu, (uint32_t)q}, k0, k1);
        const int j = (int)(((uint64_t)r.x * (uint64_t)(q + 1)) >> 32);
        const int t = cols[q];
        cols[q] = cols[j];
        cols[j] = t;
      }
      for (int k = 1; k <= n; ++k) {
        if (k >= kSubMinK)
          sub_perms_lanes(k, U, m, rows, cols, sub);
        else
          sub_perms_all(k, U, m, rows, cols, sub);
        double W = 0;
        for (int i = 0; i < m; ++i) {
          cplx z = 0;
          for (int l = 0; l < k; ++l) z += U[i * m + cols[l]] * sub[l];
          w[i] = creal(z) * creal(z) + cimag(z) * cimag(z);
          W += w[i];
        }
        const u4 r = philox((u4){slo, shi, (uint32_t)k, 0u}, k0, k1);
        const uint64_t v = ((uint64_t)(r.x >> 5) << 26) | (uint64_t)(r.y >> 6);
        const double target = (double)v * (1.0 / 9007199254740992.0) * W;
        double run = 0;
        int pick = -1, last_pos = 0;
        for (int i = 0; i < m; ++i) {
          if (w[i] > 0) last_pos = i;
          run += w[i];
          if (run > target) {
            pick = i;
            break;
          }
        }
        rows[k - 1] = pick >= 0 ? pick : last_pos;
      }
      int32_t* o = out + s * m;
      for (int i = 0; i < m; ++i) o[i] = 0;
      for (int k = 0; k < n; ++k) o[rows[k]]++;
    }
    free(w);
  }
}

/* Gurvits estimates of a batch of matrices (the CPU baseline of NaiveApprox): one OpenMP task
 * per (matrix, 256 draws), the draws' signs from the same Philox counters as oracle_gurvits
 * (draw k of matrix b has index firsts[b] + k); a draw's column sums y_j = sum_i x_i a_ij run
 * row by row over contiguous real and imaginary arrays (vectorisable over j), the product of
 * the n sums in four chains.  Each task's terms are added with Neumaier compensation and the
 * tasks of a matrix in order, so results do not depend on the thread count. */
enum { kGurvitsTask = 256 };

__attribute__((optimize("fp-contract=fast")))
void oracle_gurvits_batch_fast(const double* mats, const int64_t* offs, const int32_t* sizes, int count,
                               int64_t iterations, uint64_t seed, const uint64_t* firsts, double* out) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const int64_t per = (iterations + kGurvitsTask - 1) / kGurvitsTask;
  double* part = (double*)malloc(sizeof(double) * 4 * (size_t)(per * count > 0 ? per * count : 1));
#pragma omp parallel
  {
    double* buf = (double*)malloc(sizeof(double) * (2 * 64 * 64 + 4 * 64));
    double *ar = buf, *ai = buf + 64 * 64, *yr = ai + 64 * 64, *yi = yr + 64;
    int cur = -1;
#pragma omp for schedule(dynamic, 1)
    for (int64_t q = 0; q < per * count; ++q) {
      const int b = (int)(q / per), n = sizes[b];
      if (b != cur) {
        const double* a = mats + 2 * offs[b];
        for (int e = 0; e < n * n; ++e) {
          ar[e] = a[2 * e];
          ai[e] = a[2 * e + 1];
        }
        cur = b;
      }
      const int64_t d0 = (q % per) * kGurvitsTask;
      const int64_t d1 = d0 + kGurvitsTask < iterations ? d0 + kGurvitsTask : iterations;
      double sr = 0, cr = 0, si = 0, ci = 0;
      for (int64_t k = d0; k < d1; ++k) {
        const uint64_t idx = firsts[b] + (uint64_t)k;
        const u4 r = philox((u4){(uint32_t)idx, (uint32_t)(idx >> 32), 0x67757276u, 0u}, k0, k1);
        const uint64_t bits = (uint64_t)r.x | ((uint64_t)r.y << 32);
        for (int j = 0; j < n; ++j) yr[j] = yi[j] = 0;
        for (int i = 0; i < n; ++i) {
          const double sg = ((bits >> i) & 1) ? -1.0 : 1.0;
          const double* xr = ar + i * n;
          const double* xi = ai + i * n;
          for (int j = 0; j < n; ++j) {
            yr[j] += sg * xr[j];
            yi[j] += sg * xi[j];
          }
        }
        double pr[4] = {1, 1, 1, 1}, pi[4] = {0, 0, 0, 0};
        int j = 0;
        for (; j + 4 <= n; j += 4)
          for (int c = 0; c < 4; ++c) {
            const double x = pr[c], y = pi[c];
            pr[c] = x * yr[j + c] - y * yi[j + c];
            pi[c] = x * yi[j + c] + y * yr[j + c];
          }
        for (; j < n; ++j) {
          const double x = pr[0], y = pi[0];
          pr[0] = x * yr[j] - y * yi[j];
          pi[0] = x * yi[j] + y * yr[j];
        }
        const double r01 = pr[0] * pr[1] - pi[0] * pi[1], i01 = pr[0] * pi[1] + pi[0] * pr[1];
        const double r23 = pr[2] * pr[3] - pi[2] * pi[3], i23 = pr[2] * pi[3] + pi[2] * pr[3];
        double tr = r01 * r23 - i01 * i23, ti = r01 * i23 + i01 * r23;
        if (__builtin_popcountll(bits & (n == 64 ? ~0ull : ((1ull << n) - 1))) & 1) {
          tr = -tr;
          ti = -ti;
        }
        neumaier(&sr, &cr, tr);
        neumaier(&si, &ci, ti);
      }
      part[4 * q] = sr;
      part[4 * q + 1] = cr;
      part[4 * q + 2] = si;
      part[4 * q + 3] = ci;
    }
    free(buf);
  }
  for (int b = 0; b < count; ++b) {
    double sr = 0, cr = 0, si = 0, ci = 0;
    for (int64_t t = 0; t < per; ++t) {
      const double* x = part + 4 * (b * per + t);
      neumaier(&sr, &cr, x[0]);
      neumaier(&sr, &cr, x[1]);
      neumaier(&si, &ci, x[2]);
      neumaier(&si, &ci, x[3]);
    }
    out[2 * b] = (sr + cr) / (double)iterations;
    out[2 * b + 1] = (si + ci) / (double)iterations;
  }
  free(part);
}

/* Host-tuned SLOS (FP64).  Ranks in descending-lex order are sum_i G[i][R_i], R_i the
 * photons after mode i and G[i][r] = C(m - i + r - 2, r - 1) (0 for r = 0), so removing a
 * photon from mode j lowers the rank by sum_{i<j} (G[i][R_i] - G[i][R_i - 1]) and adding
 * one raises it by sum_{i<j} (G[i][R_i + 1] - G[i][R_i]): one O(m) pass per state gives
 * the ranks of all its parents (or children), with no per-lookup rank computation.  Each
 * OpenMP thread walks a contiguous rank range in order (one unrank per range, then
 * fock_next).  Same sums as slos_layer, in the same order per state. */
typedef struct {
  int m, n;
  uint64_t* g; /* g[i * (n + 2) + r], r = 0..n + 1 */
} RankTable;

static RankTable rank_table(int m, int n) {
  RankTable t = {m, n, (uint64_t*)malloc(sizeof(uint64_t) * m * (n + 2))};
  for (int i = 0; i < m; ++i)
    for (int r = 0; r <= n + 1; ++r) t.g[i * (n + 2) + r] = r > 0 ? fock_count(m - i, r - 1) : 0;
  return t;
}

enum { kSlosRange = 8192 };

static void slos_layer_fast(const RankTable* T, int k, const cplx* U, int mk, const cplx* prev, cplx* cur) {
  const int m = T->m, w = T->n + 2;
  const int64_t nc = (int64_t)fock_count(m, k);
  const int64_t nr = (nc + kSlosRange - 1) / kSlosRange;
#pragma omp parallel
  {
    int* s = (int*)malloc(sizeof(int) * m);
    int* R = (int*)malloc(sizeof(int) * m);
#pragma omp for schedule(dynamic, 1)
    for (int64_t q = 0; q < nr; ++q) {
      const int64_t c0 = q * kSlosRange, c1 = c0 + kSlosRange < nc ? c0 + kSlosRange : nc;
      oracle_fock_unrank(m, k, (uint64_t)c0, s);
      for (int64_t c = c0; c < c1; ++c) {
        R[m - 1] = 0;
        for (int i = m - 2; i >= 0; --i) R[i] = R[i + 1] + s[i + 1];
        cplx acc = 0;
        uint64_t d = 0;
        for (int j = 0; j < m; ++j) {
          if (s[j] > 0) acc += U[j * m + mk] * prev[(uint64_t)c - d];
          if (R[j] == 0) break;
          d += T->g[j * w + R[j]] - T->g[j * w + R[j] - 1];
        }
        cur[c] = acc;
        if (c + 1 < c1) fock_next(m, s);
      }
    }
    free(R);
    free(s);
  }
}

static double factorial_table[64];

static void fill_factorials(void) {
  factorial_table[0] = 1;
  for (int i = 1; i < 64; ++i) factorial_table[i] = factorial_table[i - 1] * i;
}

/* all n-photon layers from the input (order of _Path), into the last one */
static cplx** slos_layers_fast(int m, const cplx* U, int n, const int* order, int keep_all) {
  RankTable T = rank_table(m, n);
  cplx** L = (cplx**)calloc(n > 0 ? (size_t)n + 1 : 1, sizeof(cplx*));
  L[0] = (cplx*)malloc(sizeof(cplx));
  L[0][0] = 1;
  for (int k = 1; k <= n; ++k) {
    L[k] = (cplx*)malloc(sizeof(cplx) * fock_count(m, k));
    slos_layer_fast(&T, k, U, order[k - 1], L[k - 1], L[k]);
    if (!keep_all) {
      free(L[k - 1]);
      L[k - 1] = NULL;
    }
  }
  free(T.g);
  return L;
}

/* probabilities and amplitudes like oracle_slos, by the host-tuned layers */
int oracle_slos_fast(int m, const int* in, const double* U_, double* probs, double* amps) {
  const cplx* U = (const cplx*)U_;
  int n = 0;
  for (int i = 0; i < m; ++i) n += in[i];
  if (n < 0 || n > 63) return 1;
  fill_factorials();
  int* order = (int*)malloc(sizeof(int) * (n + 1));
  oracle_slos_order(m, in, order);
  cplx** L = slos_layers_fast(m, U, n, order, 0);
  const cplx* c = L[n];
  double pin = 1;
  for (int i = 0; i < m; ++i) pin *= factorial_table[in[i]];
  const int64_t N = (int64_t)fock_count(m, n);
  const int64_t nr = (N + kSlosRange - 1) / kSlosRange;
#pragma omp parallel
  {
    int* s = (int*)malloc(sizeof(int) * m);
#pragma omp for schedule(static)
    for (int64_t q = 0; q < nr; ++q) {
      const int64_t r0 = q * kSlosRange, r1 = r0 + kSlosRange < N ? r0 + kSlosRange : N;
      oracle_fock_unrank(m, n, (uint64_t)r0, s);
      for (int64_t r = r0; r < r1; ++r) {
        double f = 1;
        for (int i = 0; i < m; ++i) f *= factorial_table[s[i]];
        f /= pin;
        const double re = creal(c[r]), im = cimag(c[r]);
        if (probs) probs[r] = (re * re + im * im) * f;
        if (amps) {
          amps[2 * r] = re * sqrt(f);
          amps[2 * r + 1] = im * sqrt(f);
        }
        if (r + 1 < r1) fock_next(m, s);
      }
    }
    free(s);
  }
  free(L[n]);
  free(L);
  free(order);
  return 0;
}

/* dL/dU like oracle_slos_grad, by the host-tuned layers and a parallel reverse sweep (each
 * thread accumulates its parents' share of the layer's gradient column, then the shares
 * are added) */
int oracle_slos_grad_fast(int m, const int* in, const double* U_, const double* w, double* grad_) {
  const cplx* U = (const cplx*)U_;
  cplx* grad = (cplx*)grad_;
  int n = 0;
  for (int i = 0; i < m; ++i) n += in[i];
  if (n < 0 || n > 63) return 1;
  fill_factorials();
  int* order = (int*)malloc(sizeof(int) * (n + 1));
  oracle_slos_order(m, in, order);
  cplx** L = slos_layers_fast(m, U, n, order, 1);
  RankTable T = rank_table(m, n);
  const int tw = n + 2;
  for (int i = 0; i < m * m; ++i) grad[i] = 0;
  double pin = 1;
  for (int i = 0; i < m; ++i) pin *= factorial_table[in[i]];
  const int64_t N = (int64_t)fock_count(m, n);
  cplx* adj = (cplx*)malloc(sizeof(cplx) * N);
  {
    const int64_t nr = (N + kSlosRange - 1) / kSlosRange;
#pragma omp parallel
    {
      int* s = (int*)malloc(sizeof(int) * m);
#pragma omp for schedule(static)
      for (int64_t q = 0; q < nr; ++q) {
        const int64_t r0 = q * kSlosRange, r1 = r0 + kSlosRange < N ? r0 + kSlosRange : N;
        oracle_fock_unrank(m, n, (uint64_t)r0, s);
        for (int64_t r = r0; r < r1; ++r) {
          double f = 1;
          for (int i = 0; i < m; ++i) f *= factorial_table[s[i]];
          adj[r] = 2.0 * w[r] * (f / pin) * L[n][r];
          if (r + 1 < r1) fock_next(m, s);
        }
      }
      free(s);
    }
  }
  for (int k = n; k >= 1; --k) {
    const int mk = order[k - 1];
    const int64_t np = (int64_t)fock_count(m, k - 1);
    const int64_t nr = (np + kSlosRange - 1) / kSlosRange;
    cplx* pa = (cplx*)malloc(sizeof(cplx) * (np > 0 ? np : 1));
    const cplx* prev = L[k - 1];
#pragma omp parallel
    {
      int* s = (int*)malloc(sizeof(int) * m);
      int* R = (int*)malloc(sizeof(int) * m);
      cplx* gcol = (cplx*)calloc(m, sizeof(cplx));
#pragma omp for schedule(dynamic, 1)
      for (int64_t q = 0; q < nr; ++q) {
        const int64_t p0 = q * kSlosRange, p1 = p0 + kSlosRange < np ? p0 + kSlosRange : np;
        oracle_fock_unrank(m, k - 1, (uint64_t)p0, s);
        for (int64_t p = p0; p < p1; ++p) {
          R[m - 1] = 0;
          for (int i = m - 2; i >= 0; --i) R[i] = R[i + 1] + s[i + 1];
          cplx acc = 0;
          const cplx lp = conj(prev[p]);
          uint64_t d = 0;
          for (int j = 0; j < m; ++j) {
            const cplx x = adj[(uint64_t)p + d];
            acc += conj(U[j * m + mk]) * x;
            gcol[j] += lp * x;
            d += T.g[j * tw + R[j] + 1] - T.g[j * tw + R[j]];
          }
          pa[p] = acc;
          if (p + 1 < p1) fock_next(m, s);
        }
      }
#pragma omp critical
      for (int j = 0; j < m; ++j) grad[j * m + mk] += gcol[j];
      free(gcol);
      free(R);
      free(s);
    }
    free(adj);
    adj = pa;
  }
  free(adj);
  for (int k = 0; k <= n; ++k) free(L[k]);
  free(L);
  free(T.g);
  free(order);
  return 0;
}
