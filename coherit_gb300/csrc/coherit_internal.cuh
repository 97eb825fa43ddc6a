// coherit_internal.cuh -- handle state, HBM layout and shared helpers.
//
// HBM layout of the resident genotypes (both copies hold every genotype):
//   * SNP "slots": component g occupies slots [slot_start[g], slot_start[g] +
//     m_g) followed by zero padding up to a multiple of kAlign (256); the
//     total m_pad is a multiple of kAlign.  Padding slots have inv_sd = 0 and
//     never contribute.
//   * samples are padded with genotype code 0 up to n_pad (multiple of kAlign).
//   * copy S ("sample rows", operand of Z S): 2 KB blocks (sample tile st of
//     128 samples, panel p of 64 slots) at ((st * n_panels) + p) * 2048; row
//     i%128 is 16 bytes holding the 64 slots of the panel.
//   * copy T ("SNP rows", operand of Z^T V): 2 KB blocks (slot tile tt of 128
//     slots, sample chunk q of 64 samples) at ((tt * n_chunks) + q) * 2048;
//     row j%128 is 16 bytes holding the 64 samples of the chunk.
//   * inside a 16-byte row, 32-bit word w holds elements 16w + 4s + b at bits
//     8b + 2s (s, b in 0..3).  With this order, (word >> 2s) & 0x03030303
//     yields four consecutive elements, one per byte, which the decoder turns
//     into two BF16 pairs with one multiply and two byte permutes.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/coherit_gpu.h"

namespace coherit {

constexpr int kRowBytes = 16;
constexpr int kBlockRows = 128;
constexpr int kBlockBytes = kRowBytes * kBlockRows;  // 2048
constexpr int kPanel = 64;                           // slots per panel / samples per chunk
constexpr int kTile = 128;                           // rows per block
// Largest pipeline stage of the tensor-core operator (2 KB blocks along K):
// components and the sample count are padded to multiples of
// kMaxStageBlocks * 64, so that every launch's stage size divides them.
constexpr int kMaxStageBlocks = 4;
constexpr int kAlign = kPanel * kMaxStageBlocks;  // 256, a multiple of kTile
// Centring segments of the operator's first contraction: the right-hand side
// is shifted by its mean over each segment of kSegChunks sample chunks
// (4,096 samples), so the FP32 tensor-core accumulator never carries the
// running sum of a trend or an offset.
constexpr int kSegChunks = 64;
inline int64_t n_segments(int64_t n_chunks) { return (n_chunks + kSegChunks - 1) / kSegChunks; }
static_assert(kAlign % kTile == 0, "padding must hold whole 128-row tiles");

// -------------------------------------------------------------- status
void set_error(const char* fmt, ...);
// Process-wide count of kernels this library has launched.
void note_launch();
int cuda_status(cudaError_t e, const char* what);

#define CO_CUDA(call)                                         \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return ::coherit::cuda_status(_e, #call); \
  } while (0)

#define CO_CHECK(cond, code, ...)            \
  do {                                       \
    if (!(cond)) {                           \
      ::coherit::set_error(__VA_ARGS__);     \
      return (code);                         \
    }                                        \
  } while (0)

// ------------------------------------------------- within-row element order
__host__ __device__ __forceinline__ int row_word(int e) { return e >> 4; }
__host__ __device__ __forceinline__ int row_shift(int e) {
  const int r = e & 15;
  return 8 * (r & 3) + 2 * (r >> 2);
}

// ------------------------------------------------ synthetic genotype hash
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// MAF threshold of SNP s on a 2^24 scale: U(0.05, 0.5).
__host__ __device__ __forceinline__ uint32_t synth_maf_q24(uint64_t seed, int64_t s) {
  const uint64_t h = splitmix64(seed * 0xD1B54A32D192ED03ull + static_cast<uint64_t>(s));
  return 838861u + static_cast<uint32_t>((h >> 20) % 7549747ull);
}

// MAF of SNP s on a 2^24 scale, uniform on [lo, lo + span) (rare variants).
__host__ __device__ __forceinline__ uint32_t synth_maf_q24_range(uint64_t seed, int64_t s,
                                                                 uint32_t lo, uint32_t span) {
  const uint64_t h = splitmix64(seed * 0xD1B54A32D192ED03ull + static_cast<uint64_t>(s));
  return lo + static_cast<uint32_t>((h >> 20) % static_cast<uint64_t>(span));
}

// Per-SNP key of the generator: splitmix64(seed ^ s * C).
__host__ __device__ __forceinline__ uint64_t synth_snp_key(uint64_t seed, int64_t s) {
  return splitmix64(seed ^ (static_cast<uint64_t>(s) * 0x8CB92BA72F3D8DD7ull));
}

// Genotype code of sample i of the SNP with key `ks`.
__host__ __device__ __forceinline__ uint32_t synth_code_keyed(uint64_t ks, int64_t i,
                                                              uint32_t maf_q24, uint32_t miss_q24) {
  const uint64_t h = splitmix64(ks ^ (static_cast<uint64_t>(i) * 0x9E3779B97F4A7C15ull));
  const uint32_t a1 = (static_cast<uint32_t>(h) & 0xFFFFFFu) < maf_q24;
  const uint32_t a2 = (static_cast<uint32_t>(h >> 24) & 0xFFFFFFu) < maf_q24;
  if (miss_q24 != 0u && static_cast<uint32_t>(h >> 48) * 256u < miss_q24) return 3u;
  return a1 + a2;
}

// Genotype code of (sample i, SNP s): 0/1/2 allele count, 3 missing.
__host__ __device__ __forceinline__ uint32_t synth_code(uint64_t seed, int64_t s, int64_t i,
                                                        uint32_t maf_q24, uint32_t miss_q24) {
  const uint64_t key = synth_snp_key(seed, s) ^ (static_cast<uint64_t>(i) * 0x9E3779B97F4A7C15ull);
  const uint64_t h = splitmix64(key);
  const uint32_t a1 = (static_cast<uint32_t>(h) & 0xFFFFFFu) < maf_q24;
  const uint32_t a2 = (static_cast<uint32_t>(h >> 24) & 0xFFFFFFu) < maf_q24;
  if (miss_q24 != 0u && static_cast<uint32_t>(h >> 48) * 256u < miss_q24) return 3u;
  return a1 + a2;
}

// ------------------------------------------- FP32 per-SNP standardisation
// Reference FP32 standardisation from genotype counts over n_sub samples
// (geno_stream.py:1780-1792, sparse_stream.py:726-735), evaluated with
// explicitly rounded operations so that no multiply-add contraction changes
// the rounding.  n1 / n2 / n3 = het, hom-alt and missing counts.
__device__ __forceinline__ void ref_fp32_standardize(int64_t n_sub, int64_t n1, int64_t n2,
                                                     int64_t n3, float& mean, float& inv) {
  const long long cnt = static_cast<long long>(n_sub - n3);
  const long long s1 = static_cast<long long>(n1 + 2 * n2);
  const long long s2 = static_cast<long long>(n1 + 4 * n2);
  const float cnt_f = __ll2float_rn(cnt);
  const float s1_f = __ll2float_rn(s1);
  const float s2_f = __ll2float_rn(s2);
  const float denom = fmaxf(cnt_f, 1.0f);
  const float mu = __fdiv_rn(s1_f, denom);
  const float t1 = __fdiv_rn(s2_f, denom);
  const float t2 = __fmul_rn(mu, mu);
  const float var = fmaxf(__fsub_rn(t1, t2), 0.0f);
  const bool valid = (cnt_f > 0.0f) && (var > 0.0f);
  const float sd = __fsqrt_rn(fmaxf(var, 1e-6f));
  mean = mu;
  inv = valid ? __fdiv_rn(1.0f, sd) : 0.0f;
}

// ------------------------------------------------------------- handle
struct StatsSlot {
  bool used = false;
  float* mean = nullptr;        // m_pad, device
  float* inv = nullptr;         // m_pad, device
  // m_pad, device: sum over all the slot's samples of diff_ij = s1_j - cnt_j
  // * mean_j (observed allele sum minus observed count times the FP32 mean;
  // zero up to the rounding of mean_j; 0 for padding slots).
  float* dsum = nullptr;
  // n_seg x m_pad, device, segment-major (consecutive slots adjacent): the
  // same sum over the samples of each centring segment z (4,096 samples).
  float* dseg = nullptr;
  float* nseg = nullptr;  // n_seg, device: samples of the slot in each segment
  uint8_t* row_mask = nullptr;  // n_pad bytes, device; nullptr = all samples
  uint32_t* tmask = nullptr;    // n_chunks * 4 words: sample mask in row order (2 bits/sample)
  int64_t n_sub = 0;
  std::vector<double> comp_eff;
  std::vector<double> comp_atom;
  double eff_total = 0.0;
  double atom_total = 0.0;
};

// A launch configuration chosen by the autotuner for one (columns per
// launch, precision): stage size, ring depths and the grid the split-K plan
// aims for (target_mult x SMs).
struct TuneChoice {
  int wide = 0, RA = 0, RB = 0, RG = 0, target_mult = 4, cluster = 1, tiles = 1;
  float ms = 0.f;
};

struct Workspace {
  void* base = nullptr;
  size_t bytes = 0;
  int32_t k_max = 0;
  int32_t nsplit = 0;
};

}  // namespace coherit

struct coherit_geno {
  int device = 0;
  int64_t n = 0, n_pad = 0, m = 0, m_pad = 0;
  int64_t n_panels = 0, n_chunks = 0, n_stiles = 0, n_ttiles = 0;
  int32_t G = 1;
  std::vector<int64_t> comp_m;           // G
  std::vector<int64_t> comp_slot_start;  // G + 1 (slot offsets, multiples of 64)
  std::vector<int64_t> comp_snp_start;   // G + 1 (cache SNP offsets)
  int32_t* d_comp_of_slot = nullptr;     // m_pad
  int64_t* d_comp_slot_start = nullptr;  // G + 1
  int32_t* d_snp_of_slot = nullptr;      // m_pad (-1 = padding)
  int64_t* d_slot_of_snp = nullptr;      // m
  uint8_t* geno_s = nullptr;             // copy S
  uint8_t* geno_t = nullptr;             // copy T
  // missing-genotype lists (only when n_missing > 0)
  int64_t n_missing = 0;
  int64_t* d_csc_off = nullptr;  // m_pad + 1: samples with a missing genotype per slot
  int32_t* d_csc_idx = nullptr;
  int64_t* d_csr_off = nullptr;  // n_pad + 1: slots with a missing genotype per sample
  int32_t* d_csr_idx = nullptr;
  std::vector<coherit::StatsSlot> slots;
  coherit::Workspace ws;
  std::map<std::pair<int, int>, coherit::TuneChoice> tuned;  // (kp, precision)
  int* d_err = nullptr;
  int sm_count = 0;
  int smem_optin = 232448;   // max dynamic shared memory per CTA
  int smem_per_sm = 233472;  // shared memory per SM
  int64_t device_bytes = 0;
};

namespace coherit {

// Launchers implemented in the .cu files.
int build_layout_from_ref(coherit_geno* h, const uint8_t* d_packed, const int64_t* d_call_off,
                          const int32_t* d_call_pw, const int32_t* d_snp_call,
                          const int32_t* d_snp_col, cudaStream_t st);
int build_layout_synthetic(coherit_geno* h, uint64_t seed, uint32_t miss_q24, cudaStream_t st);
int build_layout_from_bed(coherit_geno* h, const uint8_t* bed_body, int64_t bps,
                          const int32_t* d_keep, const std::vector<int32_t>& slot_of_snp_host,
                          cudaStream_t st);
int build_copy_t(coherit_geno* h, cudaStream_t st);
int build_missing_lists(coherit_geno* h, cudaStream_t st);
int compute_slot_stats(coherit_geno* h, StatsSlot& s, const float* override_mean,
                       const float* override_inv, float* mean_out, float* inv_out,
                       int32_t* count_out, cudaStream_t st);
int exact_diag_launch(coherit_geno* h, const StatsSlot& s, float* out, cudaStream_t st);

// Operator launch description shared by the tensor-core and FP32 paths.
struct OpDesc {
  int mode = COHERIT_MODE_SUM;  // SUM / STACKED
  bool xtv = false;             // output X^T V (m x k) instead of Z S
  bool zxb = false;             // input is b (m x C): skip the first contraction
  int precision = COHERIT_PREC_BF16X3;
  int n_groups = 1;
  std::vector<int32_t> col_start;  // n_groups + 1
  std::vector<int32_t> slot_of_group;
  std::vector<float> comp_scale;  // n_groups * G
  std::vector<float> theta_e;     // n_groups (empty = none)
  const float* snp_weight = nullptr;  // device, cache order
  const float* V = nullptr;
  int64_t ldv = 0;
  int32_t k = 0;
  float* out = nullptr;
  int64_t ldo = 0;
};

int run_operator(coherit_geno* h, const OpDesc& d, cudaStream_t st);
int run_operator_fp32(coherit_geno* h, const OpDesc& d, cudaStream_t st);
// Tensor-core operator with its workspace in caller-provided device memory
// (`bytes` long); never allocates; rejects shapes whose workspace is larger.
int run_operator_in_scratch(coherit_geno* h, const OpDesc& d, void* scratch, size_t bytes,
                            cudaStream_t st);
int ensure_workspace(coherit_geno* h, int32_t k_max, int32_t precision);
int ensure_ws_bytes(coherit_geno* h, size_t bytes);

inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }
// AUTO resolves per launch width: E4M3 terms up to 48 columns, BF16x3 above.
constexpr int kAutoFp8MaxCols = 48;
inline int resolve_precision(int precision, int32_t k) {
  if (precision != COHERIT_PREC_AUTO) return precision;
  return round_up(k > 0 ? k : 1, 16) <= kAutoFp8MaxCols ? COHERIT_PREC_FP8X5 : COHERIT_PREC_BF16X3;
}
inline int nsplit_of(int precision) {
  if (precision == COHERIT_PREC_FP8X5) return 5;
  return precision == COHERIT_PREC_BF16X3 ? 3
         : (precision == COHERIT_PREC_BF16X2 || precision == COHERIT_PREC_FP16X2) ? 2 : 1;
}
// Operand type of the tensor-core forms: 0 BF16, 1 FP16, 2 E4M3.
constexpr int kTyBf16 = 0, kTyF16 = 1, kTyE4M3 = 2;
inline int op_type(int precision) {
  return precision == COHERIT_PREC_FP16X2 ? kTyF16
         : precision == COHERIT_PREC_FP8X5 ? kTyE4M3 : kTyBf16;
}
// Per-column power-of-two scales (FP16 and E4M3 forms).
inline bool is_scaled(int precision) { return op_type(precision) != kTyBf16; }
inline int elem_bytes(int precision) { return op_type(precision) == kTyE4M3 ? 1 : 2; }
inline bool is_tc_precision(int precision) {
  return precision >= COHERIT_PREC_BF16X3 && precision <= COHERIT_PREC_FP8X5;
}

}  // namespace coherit
