// SLOS plan state shared by the full-space kernels (slos.cu) and the masked ones
// (slos_masked.cu).  Host-side only; the kernels receive plain pointers.
#pragma once
#include <cstdint>
#include <vector>

#include "common.cuh"

// Device arrays of complex values are typed cdd but hold the plan's arithmetic: float-float
// pairs (cdd) or double2 (FP64), both 16 bytes; factor arrays (dd) hold dd or double, both
// 8 bytes.  Kernels reinterpret them through the arithmetic policies of arith.cuh.
struct pcvl_slos_plan {
  int m = 0, n = 0, B = 0;
  int prec = pcvl::kPrecFP64;    // kPrecFP64 or kPrecFloatFloat
  bool keep = false;
  std::vector<int> inputs;        // B x m input states (same photon count)
  std::vector<int32_t> col;       // n x B: input mode of photon k of entry b -> col[(k-1) * B + b]
  std::vector<uint64_t> sizes;    // layer sizes, k = 0..n (kept states for a masked plan)
  int cn_stride = 0;
  uint32_t* cn_d = nullptr;
  int32_t* col_d = nullptr;
  pcvl::dd* inv_in_d = nullptr;   // 1 / prod(in_b!) per entry
  pcvl::cdd* ucols_d = nullptr;   // [k][j][b]
  std::vector<pcvl::cdd*> layers; // keep: every layer; else layers[k % 2] ping-pong
  pcvl::cdd* adj_d[2] = {nullptr, nullptr};
  pcvl::cdd* gpart_d = nullptr;
  int gpart_blocks = 0;
  int64_t bytes = 0;
  bool forwarded = false;
  int tail_t = 0, tail_p = 0;
  uint32_t* tp_d = nullptr;       // rank_t(tau - e_j) per tail state and tail mode
  uint32_t* tc_d = nullptr;       // rank_t(tau + e_j)
  uint8_t* tocc_d = nullptr;      // occupied tail modes per tail state
  pcvl::dd* ftail_d = nullptr;    // prod tau_j! per tail state
  std::vector<uint32_t> tail_off, tstate_off, tsize;

  // Masked plan: layer k holds only the states a mask can still accept (slos_masked.cu).
  bool masked = false;
  std::vector<uint32_t*> mocc_d;    // layer k >= 1: occupied-mode bit mask of each kept state
  std::vector<uint32_t*> mpar_d;    // layer k >= 1: [e][i] index in layer k-1 of state i minus a
                                    // photon in its e-th occupied mode
  std::vector<uint32_t*> mchild_d;  // keep plans, layer k >= 1: [j][i'] index in layer k of state
                                    // i' of layer k-1 plus a photon in mode j (kNone: not kept)
  uint64_t* mrank_d = nullptr;      // kept outputs as ranks in the full n-photon space (ascending)
  pcvl::dd* mfact_d = nullptr;      // prod(out!) of each kept output

  pcvl::cdd* final_layer() const { return keep ? layers[n] : layers[n % 2]; }
};

namespace pcvl {

// shared host helpers (slos.cu)
int slos_alloc(void** p, size_t bytes, int64_t& total);
int slos_upload(void* dst, const void* src, size_t bytes);
// factors of the plan's arithmetic as 8-byte words: dd (float-float) or double (FP64)
std::vector<uint64_t> slos_factor_words(const std::vector<double>& x, int prec);
std::vector<int> slos_path_order(const std::vector<int>& input);
void slos_free_plan(pcvl_slos_plan* p);

// masked plans (slos_masked.cu)
int slos_masked_create(pcvl_slos_plan** plan, int32_t m, const int32_t* inputs, int32_t batch,
                       int32_t keep_layers, int32_t n_masks, const int8_t* digits, uint32_t at_least,
                       int32_t mask_n, int32_t precision);
int slos_masked_forward(pcvl_slos_plan* p, cudaStream_t s);
int slos_masked_finalize(pcvl_slos_plan* p, int mode, const double* w, double* out_real, double2* out_c,
                         void* seed, cudaStream_t s);
int slos_masked_backward(pcvl_slos_plan* p, const double* weights_d, double* grad_u_d, cudaStream_t s);
void slos_masked_free(pcvl_slos_plan* p);

}  // namespace pcvl
