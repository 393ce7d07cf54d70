/*
 * pcvl_gb300 — C ABI of the GB300 linear-optics kernels.
 *
 * Plain pointers and sizes only.  Every function returns 0 on success and a
 * non-zero PCVL_ERR_* code otherwise; pcvl_last_error() then gives the message
 * (per calling thread).  Device pointers (suffix _d) point to memory on the
 * current CUDA device; `stream` is a cudaStream_t (NULL = legacy default stream).
 * Complex numbers are complex128 (two interleaved doubles, re then im).
 *
 * The functions replace the calls that the reference makes into its closed
 * native library (exqalibur ~= 1.1.0); each block cites the call site.
 */
#ifndef PCVL_GB300_H
#define PCVL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCVL_OK 0
#define PCVL_ERR_ARG 1      /* bad argument: size, pointer, shape */
#define PCVL_ERR_CUDA 2     /* a CUDA runtime call failed */
#define PCVL_ERR_MEMORY 3   /* the request does not fit in device memory */
#define PCVL_ERR_TIMEOUT 4  /* a bounded device-side wait gave up */

/* Arithmetic of the permanent, SLOS and sampler kernels (`precision` arguments).
 * PCVL_PREC_FP64: FP64 precision, the reference's own arithmetic (complex128 in
 * exqalibur); the default of the Python layer.  For permanents every row sum is exact
 * (64-bit fixed point on the integer pipe), a third of each sign vector's product is
 * taken in FP64 and the rest in 64-bit block floating point on the integer pipes (62
 * significant bits), and the sums are compensated FP64 sums: no step rounds more coarsely
 * than FP64.  PCVL_PREC_FP64_DADD (permanents only): every row sum and product an FP64
 * operation, one rounding per addition.  PCVL_PREC_FLOAT_FLOAT:
 * every value an unevaluated pair of FP32 numbers (~48 significant bits) on the FP32
 * pipe, several times faster on GB300, whose FP64 rate is a small fraction of its FP32
 * rate.  PCVL_PREC_FP32: FP32 with compensated sums (sampler only). */
#define PCVL_PREC_FLOAT_FLOAT 0
#define PCVL_PREC_FP32 1
#define PCVL_PREC_FP64 2
#define PCVL_PREC_FP64_DADD 3

/* ------------------------------------------------------------------ errors */
/* Library version string, e.g. "pcvl_gb300 0.3.0 sm_103a". */
const char* pcvl_version(void);
/* Copies the calling thread's last error message into buf (NUL-terminated). */
int pcvl_last_error(char* buf, size_t len);
/* Returns to the device the scratch memory the library's pool keeps on the current
 * device (after a device synchronisation). */
int pcvl_release_workspace(void);

/* ------------------------------------------------------------------ permanents
 * Replaces xq.permanent_cx(M) (perceval/backends/_naive.py:70-71), called by
 * NaiveBackend.prob_amplitude (perceval/backends/_naive.py:46-49).
 *
 * Batched exact permanents of `count` square complex128 matrices stored row-major
 * in mats_d; matrix i starts at complex element offsets_h[i] and has size
 * sizes_h[i] (0 <= n <= 40; the permanent of the 0x0 matrix is 1).  Results go to
 * out_d[i] (complex128).  method: 0 = Glynn (sum over the 2^(n-1) sign vectors),
 * 1 = Ryser (over the 2^n column subsets).  The sign bits split into "lo" bits that
 * every thread enumerates from a shared-memory table of row-sum parts and "hi" bits
 * spread over threads and CTAs (walked in Gray-code order: exact integer updates of
 * fixed-point row sums in the FP64 default), so one large matrix uses every SM; matrices
 * are binned by size, one launch per size.  precision:
 * PCVL_PREC_FP64, PCVL_PREC_FP64_DADD or PCVL_PREC_FLOAT_FLOAT.  The matrices must not overlap in mats_d,
 * except as identical entries (same offset and size): each is rescaled in place in
 * the library's scratch at its own offsets.  offsets_h and sizes_h are host arrays.
 * Scratch comes from a stream-ordered pool per call, so concurrent calls on
 * different streams or threads are independent.
 */
int pcvl_permanent_batch(const double* mats_d, const int64_t* offsets_h, const int32_t* sizes_h,
                         int32_t count, double* out_d, int32_t method, int32_t precision, void* stream);

/* Allocation-free variant of pcvl_permanent_batch.  It has no counterpart in the
 * reference.  Some callers cannot call cudaMalloc: a plugin inside a host program
 * whose memory pool already holds the whole GPU, a latency-critical loop that must not
 * take the implicit synchronisation of an allocation, or a process whose device
 * allocations are frozen after start-up.  This entry point computes the same
 * permanents as pcvl_permanent_batch (same arguments, same results) without allocating
 * anything: its scratch is a fixed array of about 53 MB held on every GPU that loads
 * the library until the process exits.  Limits per call: at most 16384 matrices, at
 * most 3 * 2^20 complex elements spanned by offsets_h[i] + sizes_h[i]^2, at most 2^17
 * CTA partial sums.  With the built-in launch shapes the third limit is reached only
 * by batches beyond the first two; launch shapes tuned to many CTAs per SM
 * (pcvl_perm_set_tuning) can reach it with a few large matrices in each of many size
 * bins.  Larger requests are refused with PCVL_ERR_ARG and a message naming the
 * limit.  The first call on a device looks up the scratch's device address
 * (cudaGetSymbolAddress).  Every call copies its descriptors (about 24 bytes per
 * matrix) from a static host buffer.
 * Every call reuses the same scratch and
 * rewrites every part of it that it reads, so nothing needs clearing; but calls whose
 * GPU work overlaps (different streams, or different host threads without ordering)
 * race on it and must be serialised by the caller. */
int pcvl_permanent_batch_noalloc(const double* mats_d, const int64_t* offsets_h, const int32_t* sizes_h,
                                 int32_t count, double* out_d, int32_t method, int32_t precision,
                                 void* stream);

/* Monte-Carlo permanent estimates.  Replaces xq.estimate_permanent_cx(M, iterations),
 * which returns (estimate, error) to NaiveApproxBackend (perceval/backends/_naive_approx.py:52-59).
 * Matrices are packed as for pcvl_permanent_batch (0 <= n <= 40).  out_d[i]
 * (complex128) = mean of `iterations` Gurvits draws X(x) = prod_i x_i prod_j
 * (sum_i x_i a_ij), x uniform on {-1,+1}^n; err_d[i] (double) = a 99% error bound from
 * Hoeffding's inequality on the real and imaginary parts, B sqrt(4 ln 400 / iterations),
 * with B >= ||A||_2^n from a rigorous spectral-norm bound.  Draw k of matrix i uses
 * Philox4x32-10 with key = seed and counter index first_sample + i * iterations + k.
 * n = 0 gives 1 and n = 1 the element itself, both with error 0 (exact). */
int pcvl_permanent_estimate_batch(const double* mats_d, const int64_t* offsets_h, const int32_t* sizes_h,
                                  int32_t count, int64_t iterations, uint64_t seed, uint64_t first_sample,
                                  double* out_d, double* err_d, void* stream);

/* Launch-shape tuning of the permanent kernels (no reference counterpart; written by the
 * autotuner in perceval_gb300/autotune.py).  For method (0 Glynn, 1 Ryser), precision
 * (PCVL_PREC_FP64, PCVL_PREC_FP64_DADD or PCVL_PREC_FLOAT_FLOAT: each arithmetic has its
 * own table) and size n:
 * lo_bits = sign bits every thread enumerates from the shared-memory table (-1: built-in
 * min(7, max(0, F - 7)) with F the free bits), ctas_per_sm = target CTAs per SM over a
 * size bin (0: built-in 8).  Applies to later calls and plans on every device; results
 * change only by rounding.  Host-only, thread-safe. */
int pcvl_perm_set_tuning(int32_t method, int32_t precision, int32_t n, int32_t lo_bits, int32_t ctas_per_sm);
/* The effective lo bits and CTAs per SM for (method, precision, n). */
int pcvl_perm_get_tuning(int32_t method, int32_t precision, int32_t n, int32_t* lo_bits, int32_t* ctas_per_sm);

/* Permanent plans (no reference counterpart): the batch layout of pcvl_permanent_batch
 * fixed once for given sizes and offsets and executed as one CUDA graph (prepare, every
 * size bin as a concurrent branch, reduce).  Execute only swaps the input and output
 * pointers, so repeated batches of one shape (a sampler's proposal batches, a backend's
 * output lists) skip the host planning and the per-bin launches.  The tuning table is read
 * at creation.  The plan owns its device buffers; executions of one plan must be ordered
 * (one stream), and a plan is not thread-safe. */
typedef struct pcvl_perm_plan pcvl_perm_plan;

int pcvl_perm_plan_create(pcvl_perm_plan** plan, const int64_t* offsets_h, const int32_t* sizes_h,
                          int32_t count, int32_t method, int32_t precision);
int pcvl_perm_plan_execute(pcvl_perm_plan* plan, const double* mats_d, double* out_d, void* stream);
/* Device bytes the plan holds. */
int pcvl_perm_plan_bytes(const pcvl_perm_plan* plan, int64_t* bytes);
int pcvl_perm_plan_destroy(pcvl_perm_plan* plan);

/* ------------------------------------------------------------------ SLOS
 * Replaces the numeric SLOS path of perceval/backends/_slos.py:
 *   _Path._decompose / compute   (:61-102)  -> photon-addition order
 *   xq.FSArray / xq.FSMap         (:151-168) -> on-the-fly Fock ranking
 *   FSMap.compute_slos_layer      (:99)      -> pcvl_slos_forward layers
 *   prob_amplitude / all_prob / prob_distribution (:187-214, with
 *   xq.all_prob_normalize_output) -> pcvl_slos_amplitudes / pcvl_slos_probabilities
 *
 * A plan fixes (m, input state, batch): `batch` circuits share the input state and
 * each has its own m x m unitary.  Layer k holds the C(m+k-1, k) k-photon
 * coefficients of every circuit, state-major with the circuit index innermost.
 * Output index r of a circuit is the rank of the output state in descending
 * lexicographic order (|n,0,..,0> first), the order of the reference's
 * allstate_iterator.  keep_layers != 0 keeps every layer resident for
 * pcvl_slos_backward.  precision (PCVL_PREC_FP64 or PCVL_PREC_FLOAT_FLOAT) fixes the
 * arithmetic of every layer's multiply-adds and of the normalisation; a layer holds 16
 * bytes per coefficient in both.
 */
typedef struct pcvl_slos_plan pcvl_slos_plan;

int pcvl_slos_plan_create(pcvl_slos_plan** plan, int32_t m, const int32_t* input_state_h,
                          int32_t batch, int32_t keep_layers, int32_t precision);
/* Plan whose `batch` entries each have their own input state (input_states_h: batch x m,
 * host; every state must hold the same photon count).  No reference counterpart as one
 * call: it batches the per-input-state loop of Simulator._probs_svd_fast
 * (perceval/simulators/simulator.py:412-514), which calls set_input_state +
 * prob_iterator once per distinct input.  Entry b's outputs are normalised by its own
 * prod(in_b!). */
int pcvl_slos_plan_create_multi(pcvl_slos_plan** plan, int32_t m, const int32_t* input_states_h,
                                int32_t batch, int32_t keep_layers, int32_t precision);
/* Plan restricted by a mask: replaces xq.FSMask + xq.FSArray(m, k, mask) /
 * xq.FSMap(cur, prev, True) of a masked SLOSBackend (perceval/backends/_abstract_backends.py:
 * 103-137 set_mask / _init_mask; perceval/backends/_slos.py:152-166 _deploy).  Mask q is
 * digits_h[q * m .. q * m + m - 1]: a count >= 0 fixes mode i, -1 accepts any count; bit i
 * of at_least_modes makes mode i's digit a lower bound.  A state is accepted when it
 * matches one of the n_masks masks.  Layer k keeps only the k-photon states that can still
 * be completed to an accepted state of mask_n photons, so the plan's outputs are the
 * accepted n-photon states (when mask_n == n) in descending lexicographic order; their
 * count is pcvl_slos_output_count and their ranks in the full space
 * pcvl_slos_output_ranks.  Input states as pcvl_slos_plan_create_multi (batch x m, host;
 * one photon count).  Forward, probabilities, amplitudes and backward take the same
 * arguments as for a full plan, indexed by kept output. */
int pcvl_slos_plan_create_masked(pcvl_slos_plan** plan, int32_t m, const int32_t* input_states_h,
                                 int32_t batch, int32_t keep_layers, int32_t n_masks,
                                 const int8_t* digits_h, uint32_t at_least_modes, int32_t mask_n,
                                 int32_t precision);
/* Ranks of the plan's outputs in the full n-photon space (descending lexicographic order,
 * rank 0 = |n,0,..,0>), ascending: ranks_h receives pcvl_slos_output_count entries (host).
 * For a plan without mask this is 0, 1, 2, ... */
int pcvl_slos_output_ranks(const pcvl_slos_plan* plan, uint64_t* ranks_h);
int pcvl_slos_plan_destroy(pcvl_slos_plan* plan);
/* Number of output states of the plan: C(m+n-1, n), or the kept outputs of a masked plan. */
int pcvl_slos_output_count(const pcvl_slos_plan* plan, int64_t* count);
/* Device bytes the plan holds. */
int pcvl_slos_plan_bytes(const pcvl_slos_plan* plan, int64_t* bytes);
/* Propagates the input state through u_d (batch x m x m complex128, row = output
 * mode, column = input mode, circuit-major). */
int pcvl_slos_forward(pcvl_slos_plan* plan, const double* u_d, void* stream);
/* Same, with one m x m unitary u_d shared by every entry of the plan. */
int pcvl_slos_forward_shared(pcvl_slos_plan* plan, const double* u_d, void* stream);
/* pcvl_slos_forward + pcvl_slos_probabilities in one call, for callers that want only the
 * probabilities (SLOSBackend.all_prob / prob_distribution, perceval/backends/_slos.py:195-214).
 * For one circuit the last layer writes each probability directly and its coefficients are
 * not stored (no write and read-back of the largest layer); pcvl_slos_amplitudes /
 * pcvl_slos_probabilities / pcvl_slos_backward then need a pcvl_slos_forward first.
 * Results are identical to the two calls. */
int pcvl_slos_forward_probabilities(pcvl_slos_plan* plan, const double* u_d, double* probs_d, void* stream);
/* probs_d[r * batch + b] = |c|^2 * prod(out!) / prod(in!)   (float64; state-major,
 * circuit innermost) */
int pcvl_slos_probabilities(pcvl_slos_plan* plan, double* probs_d, void* stream);
/* amps_d[r * batch + b] = c * sqrt(prod(out!) / prod(in!))   (complex128) */
int pcvl_slos_amplitudes(pcvl_slos_plan* plan, double* amps_d, void* stream);
/* Adjoint of L = sum_{r,b} w[r * batch + b] * p[r, b]: writes dL/dU (torch convention,
 * dL/dRe + i dL/dIm) to grad_u_d (batch x m x m complex128).  Needs a forward with
 * keep_layers != 0 on the same plan. */
int pcvl_slos_backward(pcvl_slos_plan* plan, const double* weights_d, double* grad_u_d,
                       void* stream);

/* ------------------------------------------------------------------ SLAP
 * Replaces xq.SLAP for circuits without feed-forward (perceval/backends/_slap.py:38-80:
 * set_unitary, all_prob_ampli, all_prob, prob_distribution).  Every output of one input
 * state (m <= 4096 modes, n <= 12 photons, at most 2^36 outputs) in descending
 * lexicographic order, computed by a depth-first walk over the outputs that keeps one
 * table of 2^n photon-subset values per walker: no intermediate Fock layers.  u_d is the
 * m x m complex128 unitary (device), input_state_h the input occupation (host). */
int pcvl_slap_output_count(int32_t m, const int32_t* input_state_h, int64_t* count);
/* probs_d[r] = |Perm(U_{s_r,t})|^2 / (prod s_r! prod t!)   (count float64) */
int pcvl_slap_probabilities(const double* u_d, int32_t m, const int32_t* input_state_h, double* probs_d,
                            void* stream);
/* amps_d[r] = Perm(U_{s_r,t}) / sqrt(prod s_r! prod t!)   (count complex128) */
int pcvl_slap_amplitudes(const double* u_d, int32_t m, const int32_t* input_state_h, double* amps_d,
                         void* stream);

/* The outputs a mask keeps among the n-photon states on m modes (m <= 4096): replaces
 * iterating xq.FSArray(m, n, mask) (perceval/utils/states.py:255-290, with the mask of
 * perceval/backends/_abstract_backends.py:126-137) for any number of modes.  Mask q is
 * digits_h[q * m .. q * m + m - 1] (count >= 0, or -1 for any); at_least_h (m flags, host,
 * may be NULL) marks modes whose digit is a lower bound; mask_n is the mask's photon
 * count.  *kept receives the number of kept states; with ranks_d non-NULL (device,
 * capacity entries) their ranks in descending lexicographic order are written
 * ascending.  Synchronous. */
int pcvl_fock_mask_ranks(int32_t m, int32_t n, int32_t n_masks, const int8_t* digits_h,
                         const uint8_t* at_least_h, int32_t mask_n, uint64_t* ranks_d, int64_t capacity,
                         int64_t* kept);

/* ------------------------------------------------------------------ sampling
 * Replaces xq.Clifford2017 (perceval/backends/_clifford2017.py:36-57:
 * set_unitary / set_input_state / sample / samples).
 *
 * Draws `count` exact boson samples with the algorithm of Clifford & Clifford
 * (SODA 2018, "algorithm B"): photons are added one at a time in a uniformly random
 * order, each output mode drawn from the Laplace expansion of the k x k
 * sub-permanents.  u_d is the m x m complex128 unitary, input_state_h the input
 * occupation (host, m entries).  Sample s writes its m output counts to
 * out_counts_d[s * m .. s * m + m - 1] (int32).  Sample s uses Philox4x32-10 with
 * key (seed, 0) and counters (first_sample + s, step, draw), so results are
 * reproducible and independent of scheduling.  precision: PCVL_PREC_FLOAT_FLOAT
 * (FP64-class pairs on the FP32 pipe), PCVL_PREC_FP64 (FP64 precision: exact fixed-point
 * column sums, 64-bit block-floating products on the integer pipes, FP64 sums of the
 * terms) or PCVL_PREC_FP32 (FP32 with compensated sums); the weights and the draw are FP64
 * in every case.
 */
int pcvl_cc2017_sample(const double* u_d, int32_t m, const int32_t* input_state_h, int64_t count,
                       uint64_t seed, uint64_t first_sample, int32_t precision,
                       int32_t* out_counts_d, void* stream);
/* Samples of several input states of one photon count in one wavefront (no reference
 * counterpart as one call: it batches the per-input loop of SamplesProvider,
 * perceval/simulators/noisy_sampling_simulator.py:68-69, 120-121, which calls
 * set_input_state + samples(count) once per distinct input).  input_states_h: nstates x m
 * (host), counts_h: nstates (host).  State b's samples are rows off_b .. off_b + counts_h[b] - 1
 * of out_counts_d, off_b = counts of the states before it, and use the Philox counters of
 * samples first_sample + off_b + j: identical to pcvl_cc2017_sample per state with
 * first_sample + off_b. */
int pcvl_cc2017_sample_multi(const double* u_d, int32_t m, int32_t nstates, const int32_t* input_states_h,
                             const int64_t* counts_h, uint64_t seed, uint64_t first_sample, int32_t precision,
                             int32_t* out_counts_d, void* stream);

/* ------------------------------------------------------------------ learned proposal
 * No counterpart in the reference (its samplers have no learned part).  Kernels of
 * an autoregressive proposal network over output modes, trained on exact samples and
 * used by a Metropolised independence sampler whose acceptance uses exact permanents
 * (pcvl_permanent_batch).  bf16 arguments are __nv_bfloat16 arrays passed as void*.
 *
 * BF16 tensor-core GEMM with FP32 accumulation:
 *   C[m * ldc + n] = alpha * sum_k A(m, k) B(n, k) + beta * C[m * ldc + n]  (+ epilogue)
 *   A(m, k) = transA ? A[k * lda + m] : A[m * lda + k]
 *   B(n, k) = transB ? B[k * ldb + n] : B[n * ldb + k]
 * epilogue 0: none, 1: + bias[n], 2: + bias[n] then GELU (Cpre receives the value
 * before GELU when not null).  C (f32) and/or Cb (bf16) receive the result. */
int pcvl_gemm_bf16(const void* A, const void* B, int32_t M, int32_t N, int32_t K, int32_t lda, int32_t ldb,
                   int32_t transA, int32_t transB, float alpha, float beta, const float* bias, int32_t epilogue,
                   float* C, void* Cb, float* Cpre, int32_t ldc, void* stream);
/* op 0: GELU backward, out = x * gelu'(y) (f32 out and/or bf16 out2); op 1: f32 x ->
 * bf16 out.  n elements. */
int pcvl_mlp_elementwise(int32_t op, const void* x, const void* y, int64_t n, void* out, void* out2, void* stream);
/* out[n] = sum_m x[m * ld + n] for n < N (bias gradients). */
int pcvl_colsum(const float* x, int32_t M, int32_t N, int32_t ld, float* out, void* stream);
/* Row-wise log-softmax of R x N logits: log-probability of target[r] (logp_target),
 * optional gradient (softmax - onehot) * scale (f32 grad and/or bf16 gradb), optional
 * full log-probabilities (all_logp).  Rows with target < 0 get zero gradient. */
int pcvl_softmax_xent(const float* logits, int32_t R, int32_t N, const int32_t* target, float scale,
                      float* logp_target, float* grad, void* gradb, float* all_logp, void* stream);
/* Network input rows: h = pos_emb[k] + sum_{l<k} mode_emb[seq[s * n + l]] (bf16, D
 * columns), for every (s, k) (step < 0, row s * n + k) or for k = step (row s). */
int pcvl_bag_embed(const int32_t* seq, int32_t S, int32_t n, int32_t step, const float* mode_emb,
                   const float* pos_emb, int32_t D, void* h, void* stream);
/* Gradients of the two embedding tables from dh (f32, rows s * n + k); accumulates. */
int pcvl_bag_embed_backward(const int32_t* seq, int32_t S, int32_t n, const float* dh, int32_t D, float* dmode,
                            float* dpos, void* stream);
/* Adam step (bias-corrected, step >= 1) on f32 weights, refreshing a bf16 copy wb. */
int pcvl_adam(float* w, const float* g, float* m1, float* m2, int64_t n, float lr, float b1, float b2, float eps,
              int32_t step, void* wb, void* stream);
/* One autoregressive draw for S chains from f32 logits (S x N): seq[s * n + step] and
 * logq[s] += log-probability of the draw (Philox key seed, counter (chain0 + s, step)). */
int pcvl_sample_step(const float* logits, int32_t S, int32_t N, int32_t step, uint64_t seed, uint64_t chain0,
                     int32_t* seq, int32_t n, double* logq, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PCVL_GB300_H */
