// op_tc.cu -- the genotype operator on sm_103a tensor cores.
//
// One application  out = sum_g s_g Z_g Z_g^T V  runs as two contractions over
// the resident 2-bit genotypes (kv_impl.py:94-113 computes the same pair per
// call block, with diff materialised in FP32):
//
//   K1 (slot tiles of 128 SNPs):  T = G0^T V'           (K = samples)
//       V' = V - a_z is V shifted by its column means a_z over the request's
//       samples in each segment z of 4,096 samples, so the FP32 accumulator
//       never carries the running sum of an offset or a trend; the shift comes
//       back through the sums of diff over all samples (dsum_j, zero up to
//       the rounding of mu_j) and over each segment (dseg_jz), with a_z
//       written as the column mean abar plus d_z = a_z - abar so that a
//       constant column (d_z = 0) needs only the exact dsum_j:
//       epilogue  S_j = w_j (T_j - mu_j 1^T V' + mu_j sum_{i missing} V'_i
//                            + abar dsum_j + sum_z d_z dseg_jz)
//                 w_j = inv_sd_j^2 * s_g(j) [* snp weight]
//                 S is split into BF16 terms in the B-tile layout of K2 and
//                 r = sum_j mu_j S_j is accumulated in FP64.
//   K2 (sample tiles of 128):     out = G0 S - 1 r^T (+ theta_e V)  (K = SNPs)
//       then the sparse missing-genotype correction adds mu_j S_j back.
//
// G0 is the genotype matrix with missing codes read as 0; its entries
// {0,1,2} are exact in BF16.  Mean imputation and centring are the FP32
// rank-one terms above, so diff = G0 - mu (observed) / 0 (missing) exactly as
// in kv_impl.py:69-91.  V and S are split into up to three BF16 terms
// (hi + mid + lo) that all accumulate into one FP32 tensor-memory accumulator.
//
// Kernel anatomy: see tc_kernel.cuh.
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <vector>

#include "coherit_internal.cuh"
#include "tc_ptx.cuh"

namespace coherit {

// Pipeline configurations of the tensor-core operator, chosen per launch:
//  * StageCfg<2, 3> ("narrow"): stages of 2 blocks (K = 128), 3 decoder warp
//    sets, a 9-deep genotype ring, an A ring of 3..6 slots of 64 columns;
//    one CTA per SM.
//  * StageCfg<4, 2> ("wide"): stages of 4 blocks (K = 256), 2 decoder sets,
//    an 8-deep genotype ring, an A ring of 2..3 slots of 128 columns; half
//    the barrier round trips per K of the narrow form (at n = 50,000,
//    m = 500,000 it applies 32-48 columns in 9.0-9.8 ms against 11.3-11.7 ms).
// Ring rules: the genotype ring depth is a multiple of the decoder sets, so
// every ring slot is consumed by one set in stage order; the A ring has at
// least one slot per decoder set, so no set waits on an A slot whose previous
// use is more than one barrier phase behind (parity waits see one phase).
// The narrow form keeps at least 3 A slots: a 2-slot ring with its 3 sets
// broke the second rule (5e-3 off at n = 50,000, m = 500,000).
template <int SB_, int SETS_>
struct StageCfg {
  static constexpr int SB = SB_;        // 2 KB blocks per stage
  static constexpr int SETS = SETS_;    // decoder warp sets
  static constexpr int RG = SETS_ == 3 ? 9 : 8;  // genotype ring depth
  static constexpr int MIN_RA = SETS_ >= 3 ? 3 : SETS_;
  // Whole warpgroups: warps 0-2 copy genotypes / issue MMAs / copy B tiles,
  // warp 3 idles, warps 4.. decode.  A warp reaches only the tensor-memory
  // lanes of its SM sub-partition, which follows the hardware warp slot; a
  // CTA of whole warpgroups keeps threadIdx-derived warp % 4 equal to that
  // sub-partition even when a second CTA shares the SM.
  static constexpr int THREADS = 32 * (4 + 4 * SETS_);
  static_assert(RG % SETS_ == 0, "genotype ring depth must be a multiple of the decoder sets");
  static_assert(SB_ <= kMaxStageBlocks, "stage larger than the layout padding");
};
using CfgNarrow = StageCfg<2, 3>;
using CfgWide = StageCfg<4, 2>;
constexpr int kWarpG = 0, kWarpMMA = 1, kWarpB = 2, kWarpIdle = 3, kWarpDec0 = 4;
static_assert(kWarpDec0 % 4 == 0, "decoder sets must start on a warpgroup boundary");
// Tensor-memory A ring depth limit.  Depths up to 6 (64-column slots) are
// the configurations exercised on GB300; a 7-slot ring with a 64-column
// accumulator raised an illegal-instruction fault whose cause was not found,
// so the policy never builds one.
constexpr int kMaxRA = 6;
constexpr int kMaxRB = 16;     // B ring depth limit
constexpr int kMaxGroups = 32;
constexpr int kMaxScale = 256;
constexpr int kMaxSplitCols = 128;  // widest scaled-form launch (FP16x2: 2 x 128 <= 256)
constexpr int kBarrierBytes = 1024;

struct EpiParams {
  int n_groups, G, k, kp, nsplit, stacked, xtv, use_theta_e;
  int ty;   // operand type: kTyBf16, kTyF16 or kTyE4M3 (the last two scaled per column)
  int64_t n, m_pad, ldv, ldo;
  int32_t col_start[kMaxGroups + 1];
  const float* gmean[kMaxGroups];
  const float* ginv[kMaxGroups];
  const float* gdsum[kMaxGroups];  // m_pad sums of diff over the group slot's samples
  const float* gdseg[kMaxGroups];  // n_seg x m_pad segment sums of diff (segment-major)
  const float* gnseg[kMaxGroups];  // n_seg samples per segment of the group's slot
  int n_seg;                       // centring segments
  const uint8_t* gmask[kMaxGroups];
  float cscale[kMaxScale];
  float theta_e[kMaxGroups];
  const int32_t* comp_of_slot;
  const int32_t* snp_of_slot;
  const float* snpw;   // cache order or nullptr
  // (2 n_seg + 1) x kp: rows [0, n_seg) the segment means a_z of V over the
  // group's samples, row n_seg the column mean abar, rows n_seg + 1 + z the
  // deviations d_z = a_z - abar.
  const float* shift;
  const float* vscale; // kp: power-of-two scale of V' in K1's B tiles (1 for BF16)
  unsigned* smax;      // kp: max |S| per column (float bits), scaled forms only
  const float* cs;     // kp column sums of the shifted V
  const float* vmiss;  // m_pad x kp (shifted V over missing genotypes) or nullptr
  __nv_bfloat16* sbuf; // K1 output: S split tiles (BF16 / FP16 terms, or E4M3 bytes)
  float* sf32;         // m_pad x kp FP32 S (missing genotypes or scaled forms), else nullptr
  double* rbuf;        // (stacked ? G : 1) x kp
  float* xout;         // X^T V output (m x ldo) when xtv
  const float* V;      // K2: residual term
  float* out;          // K2 output
};

struct TcParams {
  const uint8_t* geno;
  int64_t n_chunks;    // K1: sample chunks per slot tile
  int64_t n_panels;    // K2: panels per sample tile
  const int64_t* comp_slot_start;  // device, G + 1
  const uint8_t* bsrc;
  int64_t b_chunk_bytes;
  int RB;
  int RA;
  int RG;               // genotype ring stages (<= the configuration's barrier slots)
  uint32_t bslot_bytes;
  uint32_t tmem_cols;
  uint32_t acc_cols;
  int* err;
  int64_t n_tiles;      // tiles along gridDim.x (the grid may add padding CTAs)
  int ksplit;           // CTAs along K (gridDim.z); > 1 writes partials
  float* part;          // ksplit x part_stride FP32 partials (ksplit > 1)
  int64_t part_stride;  // floats per K share: rows x kp
  int64_t part_rows;    // K2: rows per component block (n_pad)
  EpiParams e;
};

__device__ __forceinline__ int group_of(const EpiParams& e, int c) {
  int r = 0;
  while (r + 1 < e.n_groups && c >= e.col_start[r + 1]) ++r;
  return r;
}

// Decoding: a row of the genotype layout holds element 16w + 4s + b at bits
// 8b + 2s of word w, so (word >> 2s) & 0x03030303 yields four consecutive
// codes, one per byte.  t*17 + 0x40404040 turns each code c into the byte
// selector pair (c, c+4) of __byte_perm over the table bytes
// L = {0x00, 0x80, 0x00, 0x00}, H = {0x00, 0x3F, 0x40, 0x00}, i.e. the low and
// high bytes of bf16(0), bf16(1), bf16(2) and bf16(0) for code 3 (missing).
// 16 bytes = 64 codes -> 32 words of BF16 pairs in K order (word t =
// elements 2t, 2t+1).  With F16 the table holds the FP16 bytes instead:
// L = {0, 0, 0, 0}, H = {0x00, 0x3C, 0x40, 0x00} (fp16(1) = 0x3C00,
// fp16(2) = 0x4000).
template <bool F16>
__device__ __forceinline__ void decode_row(const uint4 raw, uint32_t (&a)[32]) {
  const uint32_t L = F16 ? 0u : 0x00008000u;
  const uint32_t H = F16 ? 0x00403C00u : 0x00403F00u;
  const uint32_t ws[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
  for (int w = 0; w < 4; ++w) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const uint32_t t = (ws[w] >> (2 * s)) & 0x03030303u;
      const uint32_t sel = t * 17u + 0x40404040u;
      a[8 * w + 2 * s] = __byte_perm(L, H, sel);
      a[8 * w + 2 * s + 1] = __byte_perm(L, H, sel >> 16);
    }
  }
}

// Warp sum of mu * s over the 32 lanes with FP32 arithmetic that keeps the
// rounding errors: each product as hi + lo (lo = fma(mu, s, -hi), exact), the
// lane sums by TwoSum (Knuth) with the errors carried in lo.  Returns hi + lo
// in FP64 (lane 0 adds it to the FP64 accumulator); GB300's FP64 rate is a
// small fraction of FP32, and one product per row and column fed FP64 warp
// shuffles before.
__device__ __forceinline__ double warp_sum_product(float mu, float s) {
  float hi = mu * s;
  float lo = fmaf(mu, s, -hi);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, off);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, off);
    const float sum = hi + oh;
    const float bp = sum - hi;
    const float err = (hi - (sum - bp)) + (oh - bp);
    hi = sum;
    lo = lo + ol + err;
  }
  return static_cast<double>(hi) + static_cast<double>(lo);
}

__device__ __forceinline__ void split3(float v, __nv_bfloat16& hi, __nv_bfloat16& mid,
                                       __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(hi);
  mid = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(mid);
  lo = __float2bfloat16_rn(r2);
}

// Two FP16 terms of v (already scaled into FP16's range): hi + lo carries
// 22 significant bits.
__device__ __forceinline__ void split2h(float v, __half& hi, __half& lo) {
  hi = __float2half_rn(v);
  lo = __float2half_rn(v - __half2float(hi));
}

// Power-of-two scale that maps a column whose largest magnitude is `mx` into
// [2^(top-1), 2^top): top = 14 for FP16 terms (normal, far below 65504),
// 8 for E4M3 terms (below 448, and every residual term stays below 256).
// Zero or non-finite maxima give 1.
__device__ __forceinline__ float pow2_scale(float mx, int top) {
  if (!(mx > 0.f) || !isfinite(mx)) return 1.f;
  int ex;
  frexpf(mx, &ex);  // mx = f 2^ex, f in [0.5, 1)
  const int e = max(-100, min(100, top - ex));
  return ldexpf(1.f, e);
}
__host__ __device__ __forceinline__ int scale_top(int ty) { return ty == kTyE4M3 ? 8 : 14; }

// Five E4M3 terms of x (already scaled below 256): q_0 = e4m3(x), then each
// term rounds 16 times the previous residual (exact in FP32), so
// x = sum_t q_t 16^-t + O(2^-20 |x|).
__device__ __forceinline__ void split5_e4m3(float x, uint8_t (&q)[5]) {
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const __nv_fp8_storage_t b = __nv_cvt_float_to_fp8(x, __NV_SATFINITE, __NV_E4M3);
    q[t] = static_cast<uint8_t>(b);
    const float back = __half2float(__half(__nv_cvt_fp8_to_halfraw(b, __NV_E4M3)));
    x = (x - back) * 16.f;
  }
}

// Byte offset of (column c, K index kk) inside one E4M3 term of a 64-K block
// of a B tile: core matrices of 8 columns x 16 bytes, 4 along K per 8-column
// group.
__host__ __device__ __forceinline__ int64_t btile_off8(int c, int kk) {
  return ((c >> 3) * 4 + (kk >> 4)) * 128 + (c & 7) * 16 + (kk & 15);
}

// Decoding to E4M3: codes 0, 1, 2, 3 (missing) -> bytes 0x00, 0x38 (1.0),
// 0x40 (2.0), 0x00.  16 bytes = 64 codes -> 16 words of 4 E4M3 bytes in K
// order (word 4w + s holds elements 16w + 4s .. 16w + 4s + 3).
__device__ __forceinline__ void decode_row_e4m3(const uint4 raw, uint32_t (&a)[16]) {
  const uint32_t ws[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
  for (int w = 0; w < 4; ++w) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const uint32_t t = (ws[w] >> (2 * s)) & 0x03030303u;  // one code per byte
      const uint32_t sel = (t & 0xFu) | ((t >> 4) & 0xF0u) | ((t >> 8) & 0xF00u) |
                           ((t >> 12) & 0xF000u);          // one code per nibble
      a[4 * w + s] = __byte_perm(0x00403800u, 0u, sel);
    }
  }
}

// Offset (elements) of (column c, K index kk) inside one split term of a B
// tile: K-major canonical layout, core matrices of 8 columns x 8 K values.
__host__ __device__ __forceinline__ int64_t btile_off(int c, int kk) {
  return ((c >> 3) * 8 + (kk >> 3)) * 64 + (c & 7) * 8 + (kk & 7);
}

// K1 epilogue for one 16-column chunk of slot j:
// S = w (T - mu 1^T V' + mu vmiss' + a dsum) split into BF16 terms (K2's B
// tiles), r += mu S; or the X^T V output.
__device__ __forceinline__ void epilogue_k1(const EpiParams& e, int64_t j, int c0,
                                            const float (&T)[16], int lane) {
  const int g = e.comp_of_slot[j];
  const int gi = e.stacked ? g : 0;
  const int32_t snp = e.snp_of_slot[j];
  float wsnp = 1.f;
  if (e.snpw != nullptr) wsnp = snp >= 0 ? e.snpw[snp] : 0.f;
  const int64_t pnl = j / kPanel;
  const int kk = static_cast<int>(j % kPanel);
  const int g0 = __shfl_sync(0xffffffffu, gi, 0);
  const bool uniform = __all_sync(0xffffffffu, gi == g0);
  const int64_t term = static_cast<int64_t>(e.kp) * kPanel;
  // abar dsum_j + sum_z d_z dseg_jz for the 16 columns (shifts are 0 beyond
  // k).  Columns of one request share the slot's dseg row: each run of
  // columns of one group reads it once (one load per segment, not one per
  // segment and column).
  float seg[16];
  const float* dev_rows = e.shift + static_cast<int64_t>(e.n_seg + 1) * e.kp;
#pragma unroll
  for (int i = 0; i < 16; ++i) seg[i] = 0.f;
  for (int i0 = 0; i0 < 16 && c0 + i0 < e.k;) {
    const int grp = group_of(e, c0 + i0);
    int i1 = i0 + 1;
    while (i1 < 16 && c0 + i1 < e.k && group_of(e, c0 + i1) == grp) ++i1;
    const float* ds = e.gdseg[grp] + j;
    for (int z = 0; z < e.n_seg; ++z) {
      const float d = ds[static_cast<int64_t>(z) * e.m_pad];
      const float* dr = dev_rows + static_cast<int64_t>(z) * e.kp + c0;
#pragma unroll
      for (int i = 0; i < 16; ++i)
        if (i >= i0 && i < i1) seg[i] = fmaf(dr[i], d, seg[i]);
    }
    const float dsum = e.gdsum[grp][j];
    const float* abar = e.shift + static_cast<int64_t>(e.n_seg) * e.kp + c0;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (i >= i0 && i < i1) seg[i] = fmaf(abar[i], dsum, seg[i]);
    i0 = i1;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int c = c0 + i;
    float sval = 0.f, mu = 0.f;
    if (c < e.k) {
      const int grp = group_of(e, c);
      mu = e.gmean[grp][j];
      const float iv = e.ginv[grp][j];
      const float w = (e.xtv ? iv : iv * iv) * e.cscale[grp * e.G + g] * wsnp;
      float corr = mu * e.cs[c] - seg[i];
      if (e.vmiss != nullptr) corr -= mu * e.vmiss[j * e.kp + c];
      // The B tiles held V' * vscale (a power of two): undo it exactly.
      sval = w * (T[i] * (1.f / e.vscale[c]) - corr);
    }
    if (e.xtv) {
      if (snp >= 0 && c < e.k) e.xout[static_cast<int64_t>(snp) * e.ldo + c] = sval;
      continue;
    }
    if (e.ty != kTyBf16) {
      // Scaled terms need the column's largest |S| first: keep S in FP32 and
      // its maximum (float bits order like unsigned for |S|; NaN wins);
      // k_split_s writes the B tiles and r afterwards.
      if (c < e.k) e.sf32[j * e.kp + c] = sval;
      unsigned u = __float_as_uint(fabsf(sval));
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) u = max(u, __shfl_xor_sync(0xffffffffu, u, off));
      // The column maximum only grows: skip the atomic (all warps of the
      // launch contend for kp addresses) unless this warp's maximum exceeds
      // the current one, read from L2.
      if (lane == 0 && c < e.k && u > __ldcg(&e.smax[c])) atomicMax(&e.smax[c], u);
      continue;
    }
    const int64_t base = pnl * (e.nsplit * term) + btile_off(c, kk);
    __nv_bfloat16 hi, mid, lo;
    split3(sval, hi, mid, lo);
    e.sbuf[base] = hi;
    if (e.nsplit > 1) e.sbuf[base + term] = mid;
    if (e.nsplit > 2) e.sbuf[base + 2 * term] = lo;
    if (c >= e.k) continue;
    if (e.sf32 != nullptr) e.sf32[j * e.kp + c] = sval;
    if (uniform) {
      const double v = warp_sum_product(mu, sval);
      if (lane == 0) atomicAdd(&e.rbuf[gi * e.kp + c], v);
    } else {
      atomicAdd(&e.rbuf[gi * e.kp + c], static_cast<double>(mu) * static_cast<double>(sval));
    }
  }
}

// K2 epilogue for one 16-column chunk of sample i: out = acc - r (+ theta_e V), masked.
__device__ __forceinline__ void epilogue_k2(const EpiParams& e, int64_t i, int comp, int c0,
                                            const float (&T)[16]) {
  if (i >= e.n) return;
  const int gi = e.stacked ? comp : 0;
  float* outb = e.out + static_cast<int64_t>(gi) * e.n * e.ldo;
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    const int c = c0 + t;
    if (c >= e.k) break;
    const int grp = group_of(e, c);
    float acc = T[t];
    if (e.ty != kTyBf16) acc *= 1.f / pow2_scale(__uint_as_float(e.smax[c]), scale_top(e.ty));
    float v = acc - static_cast<float>(e.rbuf[gi * e.kp + c]);
    if (e.use_theta_e) v += e.theta_e[grp] * e.V[i * e.ldv + c];
    if (e.gmask[grp] != nullptr && e.gmask[grp][i] == 0) v = 0.f;
    outb[i * e.ldo + c] = v;
  }
}

#include "tc_kernel.cuh"

// Split-K finish: T = sum of the ksplit FP32 partials of (row, 16 columns) in
// fixed order, then the K1 or K2 epilogue.  Block (32, 4): x = row within a
// 32-row group (a full warp, as epilogue_k1's reductions need), y = column
// chunk.
__global__ void __launch_bounds__(128) k_k1_finish(const float* __restrict__ part, int ksplit,
                                                    int64_t stride, EpiParams e) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * 32 + threadIdx.x;
  const int c0 = 16 * static_cast<int>(blockIdx.y * 4 + threadIdx.y);
  if (c0 >= e.kp) return;  // uniform per warp
  float T[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) T[i] = 0.f;
  for (int z = 0; z < ksplit; ++z) {
    const float4* src = reinterpret_cast<const float4*>(part + z * stride + j * e.kp + c0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 v = src[q];
      T[4 * q] += v.x; T[4 * q + 1] += v.y; T[4 * q + 2] += v.z; T[4 * q + 3] += v.w;
    }
  }
  epilogue_k1(e, j, c0, T, static_cast<int>(threadIdx.x));
}

__global__ void __launch_bounds__(128) k_k2_finish(const float* __restrict__ part, int ksplit,
                                                    int64_t stride, int64_t rows, EpiParams e) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * 32 + threadIdx.x;
  const int c0 = 16 * static_cast<int>(blockIdx.y * 4 + threadIdx.y);
  const int comp = blockIdx.z;
  if (c0 >= e.kp || i >= e.n) return;
  float T[16];
#pragma unroll
  for (int t = 0; t < 16; ++t) T[t] = 0.f;
  for (int z = 0; z < ksplit; ++z) {
    const float4* src = reinterpret_cast<const float4*>(
        part + z * stride + (static_cast<int64_t>(comp) * rows + i) * e.kp + c0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 v = src[q];
      T[4 * q] += v.x; T[4 * q + 1] += v.y; T[4 * q + 2] += v.z; T[4 * q + 3] += v.w;
    }
  }
  epilogue_k2(e, i, comp, c0, T);
}

// ------------------------------------------------------------ helper kernels

// V (n x k, fp32) -> per-chunk FP64 column sums of V (SPLIT = false), or of
// the shifted V' = V - a (SPLIT = true) together with V' split into BF16 B
// tiles for K1.  Rows outside a request's sample subset are read as zero
// (and are not shifted).
// Pass 1 also writes the per-chunk column maxima of |V| to mx_part (scaled
// forms).  Pass 2 splits V' * vscale into BF16, FP16 or E4M3 terms.
template <bool SPLIT>
__global__ void k_prep_v(const float* __restrict__ V, int64_t ldv, int64_t n, int k, int kp,
                         int nsplit, __nv_bfloat16* __restrict__ vt, double* __restrict__ cs_part,
                         float* __restrict__ mx_part, const __grid_constant__ EpiParams e) {
  extern __shared__ float tile[];  // [64][kp + 1]
  const int64_t q = blockIdx.x;
  const int ld = kp + 1;
  for (int idx = threadIdx.x; idx < kPanel * kp; idx += blockDim.x) {
    const int r = idx / kp, c = idx % kp;
    const int64_t i = q * kPanel + r;
    float v = 0.f;
    if (i < n && c < k) {
      const uint8_t* mk = e.gmask[group_of(e, c)];
      if (mk == nullptr || mk[i] != 0)
        v = SPLIT ? V[i * ldv + c] - e.shift[(q / kSegChunks) * kp + c] : V[i * ldv + c];
    }
    tile[r * ld + c] = v;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < kp; c += blockDim.x) {
    double s = 0.0;
    float mx = 0.f;
    for (int r = 0; r < kPanel; ++r) {
      s += static_cast<double>(tile[r * ld + c]);
      mx = fmaxf(mx, fabsf(tile[r * ld + c]));
    }
    cs_part[q * kp + c] = s;
    if (!SPLIT && mx_part != nullptr) mx_part[q * kp + c] = mx;
  }
  if (!SPLIT) return;
  const int cg_n = kp / 8;
  const int64_t chunk_elems = static_cast<int64_t>(nsplit) * kp * kPanel;
  if (e.ty == kTyE4M3) {
    // One byte per element: (term, 8-column group, K core, column, byte).
    uint8_t* vb = reinterpret_cast<uint8_t*>(vt);
    for (int idx = threadIdx.x; idx < chunk_elems; idx += blockDim.x) {
      const int kb = idx & 15, cr = (idx >> 4) & 7, kc = (idx >> 7) & 3;
      const int rest = idx >> 9;
      const int cg = rest % cg_n, t = rest / cg_n;
      const int c = cg * 8 + cr, kk = kc * 16 + kb;
      uint8_t qt[5];
      split5_e4m3(tile[kk * ld + c] * e.vscale[c], qt);
      vb[q * chunk_elems + idx] = qt[t];
    }
    return;
  }
  for (int idx = threadIdx.x; idx < chunk_elems; idx += blockDim.x) {
    const int kr = idx & 7, cr = (idx >> 3) & 7, kg = (idx >> 6) & 7;
    const int rest = idx >> 9;
    const int cg = rest % cg_n, t = rest / cg_n;
    const int c = cg * 8 + cr, kk = kg * 8 + kr;
    if (e.ty == kTyF16) {
      __half hi, lo;
      split2h(tile[kk * ld + c] * e.vscale[c], hi, lo);
      reinterpret_cast<__half*>(vt)[q * chunk_elems + idx] = t == 0 ? hi : lo;
    } else {
      __nv_bfloat16 hi, mid, lo;
      split3(tile[kk * ld + c], hi, mid, lo);
      vt[q * chunk_elems + idx] = t == 0 ? hi : (t == 1 ? mid : lo);
    }
  }
}

// One CTA per column: strided partial sums, then a fixed-order tree (deterministic).
__global__ void __launch_bounds__(256) k_colsum_finish(const double* __restrict__ cs_part,
                                                       int64_t n_parts, int kp,
                                                       float* __restrict__ cs) {
  __shared__ double red[256];
  const int c = blockIdx.x;
  double s = 0.0;
  for (int64_t q = threadIdx.x; q < n_parts; q += 256) s += cs_part[q * kp + c];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) cs[c] = static_cast<float>(red[0]);
}

// Segment shifts: a_zc = (sum of column c over its group's samples in
// segment z) / those samples, rounded to FP32 (any FP32 value is exact for
// the identity the K1 epilogue uses; the local mean keeps the shifted column
// and its running sums small).  One CTA per column; each segment's chunk
// partials are added in chunk order.
// For the scaled forms it also sets vscale_c = pow2_scale(max |V_c| +
// max_z |a_zc|), a bound on max |V'_c|, so that V' * vscale fits the terms.
__global__ void __launch_bounds__(256) k_shift_finish(const double* __restrict__ cs_part,
                                                      const float* __restrict__ mx_part,
                                                      int64_t n_parts, int kp,
                                                      float* __restrict__ shift,
                                                      float* __restrict__ vscale,
                                                      const __grid_constant__ EpiParams e) {
  __shared__ float redm[256];
  __shared__ double red[256];
  __shared__ double redn[256];
  const int c = blockIdx.x;
  const float* nseg = c < e.k ? e.gnseg[group_of(e, c)] : nullptr;
  // Column total and sample count (fixed-order tree), then abar.
  double tot = 0.0, cnt = 0.0;
  for (int z = threadIdx.x; z < e.n_seg; z += 256) {
    const int64_t q1 = min(n_parts, static_cast<int64_t>(z + 1) * kSegChunks);
    for (int64_t q = static_cast<int64_t>(z) * kSegChunks; q < q1; ++q) tot += cs_part[q * kp + c];
    if (nseg != nullptr) cnt += static_cast<double>(nseg[z]);
  }
  red[threadIdx.x] = tot;
  redn[threadIdx.x] = cnt;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[threadIdx.x] += red[threadIdx.x + w];
      redn[threadIdx.x] += redn[threadIdx.x + w];
    }
    __syncthreads();
  }
  const float abar = redn[0] > 0.0 ? static_cast<float>(red[0] / redn[0]) : 0.f;
  if (threadIdx.x == 0) shift[static_cast<int64_t>(e.n_seg) * kp + c] = abar;
  float mx = fabsf(abar);
  for (int z = threadIdx.x; z < e.n_seg; z += 256) {
    double s = 0.0;
    const int64_t q1 = min(n_parts, static_cast<int64_t>(z + 1) * kSegChunks);
    for (int64_t q = static_cast<int64_t>(z) * kSegChunks; q < q1; ++q) s += cs_part[q * kp + c];
    float a = abar;
    if (nseg != nullptr && nseg[z] > 0.f) a = static_cast<float>(s / static_cast<double>(nseg[z]));
    if (nseg == nullptr) a = 0.f;
    shift[z * kp + c] = a;
    shift[(static_cast<int64_t>(e.n_seg) + 1 + z) * kp + c] = a - abar;
    mx = fmaxf(mx, fabsf(a));
  }
  if (e.ty != kTyBf16) {
    float vm = 0.f;
    for (int64_t q = threadIdx.x; q < n_parts; q += 256) vm = fmaxf(vm, mx_part[q * kp + c]);
    redm[threadIdx.x] = vm;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) redm[threadIdx.x] = fmaxf(redm[threadIdx.x], redm[threadIdx.x + w]);
      __syncthreads();
    }
    const float vmax = redm[0];
    __syncthreads();
    redm[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) redm[threadIdx.x] = fmaxf(redm[threadIdx.x], redm[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) vscale[c] = pow2_scale(vmax + redm[0], scale_top(e.ty));
  } else if (threadIdx.x == 0) {
    vscale[c] = 1.f;
  }
}

// vmiss[j, c] = sum over samples i with a missing genotype at slot j of the
// shifted V'[i, c] = V[i, c] - a_c.
__global__ void k_vmiss(const int64_t* __restrict__ off, const int32_t* __restrict__ idx,
                        int64_t m_pad, const float* __restrict__ V, int64_t ldv, int64_t n, int k,
                        int kp, float* __restrict__ vmiss, const __grid_constant__ EpiParams e) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (j >= m_pad) return;
  for (int c = lane; c < kp; c += 32) {
    double s = 0.0;
    if (c < k) {
      const uint8_t* mk = e.gmask[group_of(e, c)];
      for (int64_t t = off[j]; t < off[j + 1]; ++t) {
        const int64_t i = idx[t];
        if (i < n && (mk == nullptr || mk[i] != 0))
          s += static_cast<double>(V[i * ldv + c] -
                                   e.shift[(i / (kSegChunks * kPanel)) * kp + c]);
      }
    }
    vmiss[j * kp + c] = static_cast<float>(s);
  }
}

// out[i, c] += mu_j S_j[c] over slots j where sample i's genotype is missing.
__global__ void k_rowcorr(const int64_t* __restrict__ off, const int32_t* __restrict__ idx,
                          int64_t n, const __grid_constant__ EpiParams e) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  for (int c = lane; c < e.k; c += 32) {
    const int grp = group_of(e, c);
    if (e.gmask[grp] != nullptr && e.gmask[grp][i] == 0) continue;
    const float* mean = e.gmean[grp];
    for (int64_t t = off[i]; t < off[i + 1]; ++t) {
      const int64_t j = idx[t];
      const int g = e.stacked ? e.comp_of_slot[j] : 0;
      e.out[(static_cast<int64_t>(g) * e.n + i) * e.ldo + c] += mean[j] * e.sf32[j * e.kp + c];
    }
  }
}

// b (m x C, cache order) -> S = inv_sd * b split into K2 B tiles, r = sum mu S.
// One thread per slot; the FP64 terms of r are summed across the warp first
// (one atomic per warp and column: per-slot atomics onto the k entries of r
// serialised, 12.8 ms at m = 300,000, k = 64).
__global__ void k_prep_s_from_b(const float* __restrict__ b, int64_t ldb,
                                const __grid_constant__ EpiParams e) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const bool active = j < e.m_pad;  // every lane stays for the warp reductions
  const int lane = threadIdx.x & 31;
  const int32_t snp = active ? e.snp_of_slot[j] : -1;
  const float mu = active ? e.gmean[0][j] : 0.f;
  const float iv = active ? e.ginv[0][j] : 0.f;
  const int64_t pnl = j / kPanel;
  const int kk = static_cast<int>(j % kPanel);
  for (int c = 0; c < e.kp; ++c) {
    float sval = 0.f;
    if (c < e.k && snp >= 0) sval = iv * b[static_cast<int64_t>(snp) * ldb + c];
    if (e.ty != kTyBf16) {
      // FP32 S and its column maximum; k_split_s forms the scaled tiles and r.
      if (active && c < e.k) e.sf32[j * e.kp + c] = sval;
      unsigned u = __float_as_uint(fabsf(sval));
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) u = max(u, __shfl_xor_sync(0xffffffffu, u, off));
      // The column maximum only grows: skip the atomic (all warps of the
      // launch contend for kp addresses) unless this warp's maximum exceeds
      // the current one, read from L2.
      if (lane == 0 && c < e.k && u > __ldcg(&e.smax[c])) atomicMax(&e.smax[c], u);
      continue;
    }
    if (active) {
      const int64_t base =
          pnl * (static_cast<int64_t>(e.nsplit) * e.kp * kPanel) + btile_off(c, kk);
      __nv_bfloat16 hi, mid, lo;
      split3(sval, hi, mid, lo);
      e.sbuf[base] = hi;
      if (e.nsplit > 1) e.sbuf[base + static_cast<int64_t>(e.kp) * kPanel] = mid;
      if (e.nsplit > 2) e.sbuf[base + 2 * static_cast<int64_t>(e.kp) * kPanel] = lo;
      if (c < e.k && e.sf32 != nullptr) e.sf32[j * e.kp + c] = sval;
    }
    if (c < e.k) {
      double v = static_cast<double>(mu) * static_cast<double>(sval);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0 && v != 0.0) atomicAdd(&e.rbuf[c], v);
    }
  }
}

// Scaled forms: S (FP32, m_pad x kp) -> K2's B tiles of S * tau_c in two
// FP16 or five E4M3 terms, tau_c = pow2_scale(max_j |S_jc|), and
// r = sum_j mu_j S_j in FP64
// (per component when stacked).  One thread per slot; a warp's 32 slots lie
// in one component (components start on multiples of 256 slots), checked
// before the warp reduction.
// Threads per block of k_split_s: its per-column sums of mu S are combined
// over the block's warps in shared memory before one FP64 atomic per block
// and column (one per warp and column serialised on the 48-odd addresses).
constexpr int kSplitThreads = 256;

__global__ void __launch_bounds__(kSplitThreads) k_split_s(const __grid_constant__ EpiParams e) {
  __shared__ double red[kSplitThreads / 32][kMaxSplitCols];
  __shared__ int block_g;
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const bool active = j < e.m_pad;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = active ? e.comp_of_slot[j] : 0;
  const int gi = e.stacked ? g : 0;
  if (threadIdx.x == 0) block_g = gi;
  __syncthreads();
  // One component for the whole block: sums per warp into shared memory.
  const bool block_uniform = __syncthreads_and(gi == block_g) != 0;
  const int g0 = __shfl_sync(0xffffffffu, gi, 0);
  const bool uniform = __all_sync(0xffffffffu, gi == g0);
  const int64_t pnl = j / kPanel;
  const int kk = static_cast<int>(j % kPanel);
  const int64_t term = static_cast<int64_t>(e.kp) * kPanel;  // elements of one term
  const int top = scale_top(e.ty);
  // The row's S values in 16-byte loads (kp is a multiple of 16).
  const float4* srow = reinterpret_cast<const float4*>(e.sf32 + (active ? j : 0) * e.kp);
  float4 sv4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int c = 0; c < e.kp; ++c) {
    float sval = 0.f, mu = 0.f;
    if ((c & 3) == 0 && active) sv4 = srow[c >> 2];
    if (active && c < e.k) {
      const int q = c & 3;
      sval = q == 0 ? sv4.x : q == 1 ? sv4.y : q == 2 ? sv4.z : sv4.w;
      mu = e.gmean[group_of(e, c)][j];
    }
    if (active) {
      const float tau = c < e.k ? pow2_scale(__uint_as_float(e.smax[c]), top) : 1.f;
      if (e.ty == kTyE4M3) {
        uint8_t q[5];
        split5_e4m3(sval * tau, q);
        uint8_t* sb = reinterpret_cast<uint8_t*>(e.sbuf) + pnl * (5 * term) + btile_off8(c, kk);
#pragma unroll
        for (int t = 0; t < 5; ++t) sb[t * term] = q[t];
      } else {
        __half hi, lo;
        split2h(sval * tau, hi, lo);
        __half* sb = reinterpret_cast<__half*>(e.sbuf);
        const int64_t base = pnl * (2 * term) + btile_off(c, kk);
        sb[base] = hi;
        sb[base + term] = lo;
      }
    }
    if (c >= e.k) continue;
    if (block_uniform) {
      const double v = warp_sum_product(mu, sval);
      if (lane == 0) red[warp][c] = v;
    } else if (uniform) {
      const double v = warp_sum_product(mu, sval);
      if (lane == 0 && v != 0.0) atomicAdd(&e.rbuf[gi * e.kp + c], v);
    } else {
      const double v = static_cast<double>(mu) * static_cast<double>(sval);
      if (v != 0.0) atomicAdd(&e.rbuf[gi * e.kp + c], v);
    }
  }
  if (block_uniform) {
    __syncthreads();
    for (int c = threadIdx.x; c < e.k; c += blockDim.x) {
      double t = 0.0;
#pragma unroll
      for (int w = 0; w < kSplitThreads / 32; ++w) t += red[w][c];
      if (t != 0.0) atomicAdd(&e.rbuf[block_g * e.kp + c], t);
    }
  }
}

// ------------------------------------------------------------------ launcher

// Widest right-hand-side block of one launch: two B ring slots (one stage of
// all split terms each) next to the genotype ring must fit the 227 KB of
// dynamic shared memory, and N <= 256.
// The split terms always sit side by side in N (nsplit * kp <= 256):
// accumulating them one after another into one accumulator loses accuracy
// on long chains (measured 6.5e-4 relative at n = 50,000, m = 500,000).
static inline int max_kp_for(const coherit_geno* h, int nsplit, int eb) {
  const int budget =
      h->smem_optin - 4096 - kBarrierBytes - CfgNarrow::RG * CfgNarrow::SB * kBlockBytes;
  const int per_col = 2 * CfgNarrow::SB * nsplit * kPanel * eb;
  return std::min((256 / nsplit) / 16 * 16, (budget / per_col) / 16 * 16);
}

// Split K.  Longest chain one accumulator takes: 65,536 K values (4,096 MMAs
// of K = 16; 512 two-block or 256 four-block stages).  Measured on GB300 at
// n = 50,000: K2 chains over 62,500 SNPs stay within 2e-6 relative of FP64,
// over 500,000 SNPs 4.5e-5; chains of 131,072 (512 four-block stages) let a
// served PCG at n = 200,000, m = 600,000 stall at 1.4e-5 against a 1e-5
// tolerance.  Short problems are split further, down to 2,048 K values a
// share, until the grid holds about two waves.
constexpr int64_t kMaxChainK = 65536;
constexpr int64_t kMinShareK = 2048;

static int split_count(int64_t stages, int64_t ctas, int64_t target_ctas, int sb) {
  const int64_t max_stages = kMaxChainK / (kPanel * sb);
  const int64_t min_stages = std::max<int64_t>(1, kMinShareK / (kPanel * sb));
  int64_t P = std::max<int64_t>(1, (stages + max_stages - 1) / max_stages);
  if (ctas * P < target_ctas) {
    const int64_t want = (target_ctas + ctas - 1) / ctas;
    P = std::max(P, std::min(want, stages / min_stages));
  }
  return static_cast<int>(std::min<int64_t>(P, 1024));
}

struct SplitPlan {
  int k1, k2;     // K shares of K1 and of K2
  int64_t nr;     // K2 component blocks (G when stacked, else 1)
};

// K shares of one launch whose stages hold `sb` blocks and whose CTAs own
// `tiles` row tiles each.
static SplitPlan split_plan(const coherit_geno* h, bool stacked, int64_t target_ctas, int sb,
                            int tiles) {
  SplitPlan s;
  s.nr = stacked ? h->G : 1;
  s.k1 = split_count(h->n_chunks / sb, (h->n_ttiles + tiles - 1) / tiles, target_ctas, sb);
  int64_t stages2 = h->n_panels / sb;
  if (stacked) {
    stages2 = 0;
    for (int g = 0; g < h->G; ++g)
      stages2 = std::max<int64_t>(
          stages2, (h->comp_slot_start[g + 1] - h->comp_slot_start[g]) / kPanel / sb);
  }
  s.k2 = split_count(stages2, (h->n_stiles + tiles - 1) / tiles * s.nr, target_ctas, sb);
  return s;
}

// Grid size that fills about two waves of the operator kernel.
// Grid size the split-K plan fills: about two waves (4 x SMs), or the
// autotuner's choice for this width and precision.  Partial buffers are sized
// for the largest multiple the tuner tries.
constexpr int kDefaultTargetMult = 4;
constexpr int kMaxTargetMult = 8;
static int64_t target_ctas(const coherit_geno* h, int mult = kDefaultTargetMult) {
  return static_cast<int64_t>(mult) * std::max(h->sm_count, 1);
}
static int64_t target_ctas_for(const coherit_geno* h, int kp, int precision) {
  const auto it = h->tuned.find({kp, precision});
  return target_ctas(h, it == h->tuned.end() ? kDefaultTargetMult : it->second.target_mult);
}

struct WsLayout {
  size_t vt, sbuf, cs_part, mx_part, cs, shift, vscale, smax, rbuf, vmiss, sf32, part, total;
};

static size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

// Split-K partial buffer (floats per column): the larger of K1's and K2's,
// over both output modes.  K1's partials are consumed before K2 runs.
static int64_t part_rows_needed(const coherit_geno* h) {
  int64_t rows = 0;
  for (int q = 0; q < 8; ++q) {
    const bool stacked = (q & 1) != 0;
    const int sb = (q & 2) ? CfgWide::SB : CfgNarrow::SB;
    const int tiles = (q & 4) ? 2 : 1;
    const SplitPlan s = split_plan(h, stacked, target_ctas(h, kMaxTargetMult), sb, tiles);
    if (s.k1 > 1) rows = std::max<int64_t>(rows, s.k1 * h->m_pad);
    if (s.k2 > 1) rows = std::max<int64_t>(rows, s.k2 * s.nr * h->n_pad);
  }
  return rows;
}

static WsLayout ws_layout(const coherit_geno* h, int kp, int precision) {
  const int nsplit = nsplit_of(precision);
  const int eb = elem_bytes(precision);
  const bool f16 = is_scaled(precision);
  WsLayout L;
  size_t off = 0;
  L.vt = off;
  off = align256(off + static_cast<size_t>(h->n_chunks) * nsplit * kp * kPanel * eb);
  L.sbuf = off;
  off = align256(off + static_cast<size_t>(h->n_panels) * nsplit * kp * kPanel * eb);
  L.cs_part = off;
  off = align256(off + static_cast<size_t>(h->n_chunks) * kp * 8);
  L.mx_part = off;
  if (f16) off = align256(off + static_cast<size_t>(h->n_chunks) * kp * 4);
  L.cs = off;
  off = align256(off + static_cast<size_t>(kp) * 4);
  L.shift = off;
  off = align256(off + static_cast<size_t>(2 * n_segments(h->n_chunks) + 1) * kp * 4);
  L.vscale = off;
  off = align256(off + static_cast<size_t>(kp) * 4);
  L.smax = off;
  off = align256(off + static_cast<size_t>(kp) * 4);
  L.rbuf = off;
  off = align256(off + static_cast<size_t>(h->G) * kp * 8);
  L.vmiss = off;
  L.sf32 = off;
  if (h->n_missing > 0) off = align256(off + static_cast<size_t>(h->m_pad) * kp * 4);
  L.sf32 = off;
  if (h->n_missing > 0 || f16) off = align256(off + static_cast<size_t>(h->m_pad) * kp * 4);
  L.part = off;
  off = align256(off + static_cast<size_t>(part_rows_needed(h)) * kp * 4);
  L.total = off;
  return L;
}

int ensure_ws_bytes(coherit_geno* h, size_t bytes) {
  if (h->ws.base != nullptr && h->ws.bytes >= bytes) return COHERIT_OK;
  if (h->ws.base != nullptr) {
    // The old buffer may still be read by queued work.
    CO_CUDA(cudaDeviceSynchronize());
    cudaFree(h->ws.base);
    h->ws = Workspace();
  }
  CO_CUDA(cudaMalloc(&h->ws.base, bytes));
  h->ws.bytes = bytes;
  return COHERIT_OK;
}

int ensure_workspace(coherit_geno* h, int32_t k_max, int32_t precision) {
  const int kp = static_cast<int>(round_up(std::max(k_max, 1), 16));
  const WsLayout L = ws_layout(h, kp, precision);
  return ensure_ws_bytes(h, L.total);
}

static int fill_epi(coherit_geno* h, const OpDesc& d, int kp, int nsplit, EpiParams& e) {
  memset(&e, 0, sizeof(e));
  CO_CHECK(d.n_groups >= 1 && d.n_groups <= kMaxGroups, COHERIT_E_SHAPE,
           "number of requests per launch must be in [1, %d]", kMaxGroups);
  CO_CHECK(d.n_groups * h->G <= kMaxScale, COHERIT_E_SHAPE,
           "requests x components must not exceed %d", kMaxScale);
  e.n_groups = d.n_groups;
  e.G = h->G;
  e.k = d.k;
  e.kp = kp;
  e.nsplit = nsplit;
  e.stacked = d.mode == COHERIT_MODE_STACKED ? 1 : 0;
  e.xtv = d.xtv ? 1 : 0;
  e.ty = op_type(d.precision);
  e.n = h->n;
  e.m_pad = h->m_pad;
  e.n_seg = static_cast<int>(n_segments(h->n_chunks));
  e.ldv = d.ldv;
  e.ldo = d.ldo;
  for (int r = 0; r <= d.n_groups; ++r) e.col_start[r] = d.col_start[r];
  for (int r = 0; r < d.n_groups; ++r) {
    const int s = d.slot_of_group[r];
    CO_CHECK(s >= 0 && s < static_cast<int>(h->slots.size()) && h->slots[s].used,
             COHERIT_E_INDEX, "stats slot %d is not initialised", s);
    e.gmean[r] = h->slots[s].mean;
    e.ginv[r] = h->slots[s].inv;
    e.gdsum[r] = h->slots[s].dsum;
    e.gdseg[r] = h->slots[s].dseg;
    e.gnseg[r] = h->slots[s].nseg;
    e.gmask[r] = h->slots[s].row_mask;
    for (int g = 0; g < h->G; ++g) e.cscale[r * h->G + g] = d.comp_scale[r * h->G + g];
    e.theta_e[r] = d.theta_e.empty() ? 0.f : d.theta_e[r];
  }
  e.use_theta_e = d.theta_e.empty() ? 0 : 1;
  e.comp_of_slot = h->d_comp_of_slot;
  e.snp_of_slot = h->d_snp_of_slot;
  e.snpw = d.snp_weight;
  e.V = d.V;
  e.out = d.out;
  e.xout = d.out;
  return COHERIT_OK;
}

struct TcLaunchCfg {
  bool wide;   // StageCfg<4, 2> instead of StageCfg<2, 3>
  int sb;      // blocks per stage of that configuration
  int cluster; // CTAs per cluster sharing each B tile (1 or 2)
  int tiles;   // row tiles per CTA (1, or 2 with two MMA-issuing threads)
  int RG;      // genotype ring stages
  int RB, RA;
  bool side;
  uint32_t bslot;
  uint32_t tmem_cols, acc_cols;
  size_t smem;
};

// Requested launch shape: wide -1 policy, 0 two-block stages, 1 four-block
// stages (if their rings fit); ring depths 0 = largest that fits (genotype
// ring: the configuration's full depth), clamped to what fits tensor
// memory, shared memory and the barrier arrays; cluster 0 = policy.
struct LaunchReq {
  int wide = -1, RA = 0, RB = 0, RG = 0, cluster = 0, tiles = 0;
};

static LaunchReq req_of(const TuneChoice& t) {
  LaunchReq r;
  r.wide = t.wide;
  r.RA = t.RA;
  r.RB = t.RB;
  r.RG = t.RG;
  r.cluster = t.cluster;
  r.tiles = t.tiles;
  return r;
}

// CTAs per cluster and row tiles per CTA of the fixed policy (no tuned
// choice); two tiles only where their accumulators and rings fit.
constexpr int kDefaultCluster = 1;
constexpr int kDefaultTiles = 1;

// Accumulator: NSPLIT*kp columns, the split terms side by side in N (one MMA
// per K step, N <= 256).  The A ring takes the remaining tensor-memory
// columns.  Blocks of <= 16 columns use the narrow form; wider blocks use the
// wide form where its B ring (>= 2 stages) fits shared memory, else the
// narrow form; always one CTA per SM, which allocates all 512 tensor-memory
// columns so no second CTA can share the SM.
static TcLaunchCfg tc_config_policy(const coherit_geno* h, int kp, int precision,
                                    const LaunchReq& rq) {
  const int nsplit = nsplit_of(precision);
  const int eb = elem_bytes(precision);
  // Tensor-memory columns of one 64-K block of A (E4M3: one byte per code).
  const uint32_t acols = op_type(precision) == kTyE4M3 ? 16u : 32u;
  TcLaunchCfg c;
  c.cluster = rq.cluster == 1 || rq.cluster == 2 ? rq.cluster : kDefaultCluster;
  c.side = nsplit > 1 && nsplit * kp <= 256;
  const int acc = c.side ? nsplit * kp : kp;
  c.acc_cols = static_cast<uint32_t>(round_up(acc, 32));
  const size_t cap = static_cast<size_t>(h->smem_optin);
  auto ring_g = [&](int sets, int full) {
    return rq.RG >= sets && rq.RG <= full && rq.RG % sets == 0 ? rq.RG : full;
  };
  const int want_tiles = rq.tiles == 1 || rq.tiles == 2 ? rq.tiles : kDefaultTiles;
  // Two tiles per CTA where both accumulators, an A ring of at least the
  // minimum depth for both tiles and the doubled genotype slots fit; else one.
  for (int tiles = want_tiles; tiles >= 1; --tiles) {
    c.tiles = tiles;
    const uint32_t acc_all = static_cast<uint32_t>(tiles) * c.acc_cols;
    if (acc_all >= 512u) continue;
    if (rq.wide != 0) {
      // Four-block stages (half the barrier round trips per K of two-block
      // stages) wherever their rings fit: at one CTA per SM they apply 16
      // columns faster than two-block stages (n = 50,000, m = 500,000: k = 32
      // in 10.5 ms against k = 16 in 12.7 ms with two-block stages).
      const int rg = ring_g(CfgWide::SETS, CfgWide::RG);
      const uint32_t slot = acols * CfgWide::SB * tiles;
      const uint32_t bslot = static_cast<uint32_t>(CfgWide::SB) * nsplit * kp * kPanel * eb;
      const size_t fixed =
          kBarrierBytes + static_cast<size_t>(rg) * CfgWide::SB * kBlockBytes * tiles;
      int ra = std::min<int>(kMaxRA, static_cast<int>((512u - acc_all) / slot));
      if (rq.RA > 0) ra = std::min(ra, std::max(rq.RA, CfgWide::MIN_RA));
      if (acc_all + CfgWide::MIN_RA * slot <= 512u && ra >= CfgWide::MIN_RA &&
          fixed + 2 * static_cast<size_t>(bslot) <= cap - 4096) {
        c.wide = true;
        c.sb = CfgWide::SB;
        c.RG = rg;
        c.tmem_cols = 512;
        c.RA = ra;
        c.bslot = bslot;
        int rb = static_cast<int>((cap - 4096 - fixed) / bslot);
        if (rq.RB > 0) rb = std::min(rb, rq.RB);
        c.RB = std::max(2, std::min(kMaxRB, rb));
        c.smem = fixed + static_cast<size_t>(c.RB) * bslot;
        return c;
      }
    }
    c.wide = false;
    c.sb = CfgNarrow::SB;
    c.RG = ring_g(CfgNarrow::SETS, CfgNarrow::RG);
    const uint32_t slot_cols = acols * CfgNarrow::SB * tiles;
    c.bslot = static_cast<uint32_t>(CfgNarrow::SB) * nsplit * kp * kPanel * eb;
    const size_t fixed =
        kBarrierBytes + static_cast<size_t>(c.RG) * CfgNarrow::SB * kBlockBytes * tiles;
    if (tiles > 1 && (acc_all + CfgNarrow::MIN_RA * slot_cols > 512u ||
                      fixed + 2 * static_cast<size_t>(c.bslot) > cap - 4096))
      continue;
    // One CTA per SM for every width: all 512 tensor-memory columns.  Layouts
    // with two CTAs per SM returned a few wrong rows under split K (a whole
    // lane quarter of a tile) even with CTAs of whole warpgroups.
    c.tmem_cols = 512;
    c.RA = std::min<int>(kMaxRA, static_cast<int>((512u - acc_all) / slot_cols));
    if (rq.RA > 0) c.RA = std::min(c.RA, std::max(rq.RA, CfgNarrow::MIN_RA));
    int rb = static_cast<int>((cap - 4096 - fixed) / c.bslot);
    if (rq.RB > 0) rb = std::min(rb, rq.RB);
    rb = std::max(2, std::min(kMaxRB, rb));
    while (rb > 2 && fixed + static_cast<size_t>(rb) * c.bslot > cap) --rb;
    c.RB = rb;
    c.smem = fixed + static_cast<size_t>(rb) * c.bslot;
    // One CTA per SM: pad the shared-memory request until a second CTA cannot
    // fit (it would block in tcgen05.alloc).
    const size_t sm_bytes = static_cast<size_t>(h->smem_per_sm);
    while (static_cast<int>(sm_bytes / (c.smem + 1024)) > 1 && c.smem + 4096 <= cap)
      c.smem += 4096;
    return c;
  }
  return c;  // not reached: one tile always fits (max_kp_for)
}

// Launch configuration: the autotuner's choice for (kp, precision) when there
// is one, else the fixed policy.
static TcLaunchCfg tc_config(const coherit_geno* h, int kp, int precision) {
  const auto it = h->tuned.find({kp, precision});
  if (it != h->tuned.end()) return tc_config_policy(h, kp, precision, req_of(it->second));
  return tc_config_policy(h, kp, precision, LaunchReq());
}

template <bool IS_K1, class Cfg, int CL, int TILES>
static int launch_tc_cfg(int nsplit, int ty, bool side, dim3 grid, size_t smem,
                         cudaStream_t st, const TcParams& p) {
  auto go = [&](auto kern) -> int {
    CO_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)));
    if constexpr (CL == 1) {
      kern<<<grid, Cfg::THREADS, smem, st>>>(p);
    } else {
      cudaLaunchConfig_t lc = {};
      lc.gridDim = grid;
      lc.blockDim = dim3(Cfg::THREADS);
      lc.dynamicSmemBytes = smem;
      lc.stream = st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = CL;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      lc.attrs = at;
      lc.numAttrs = 1;
      CO_CUDA(cudaLaunchKernelEx(&lc, kern, p));
    }
    note_launch();
    CO_CUDA(cudaGetLastError());
    return COHERIT_OK;
  };
  if (ty == kTyF16) {
    CO_CHECK(nsplit == 2 && side, COHERIT_E_SHAPE, "FP16 terms must fit side by side (2 kp <= 256)");
    return go(k_tc_op<IS_K1, 2, true, Cfg, kTyF16, CL, TILES>);
  }
  if (ty == kTyE4M3) {
    CO_CHECK(nsplit == 5 && side, COHERIT_E_SHAPE, "E4M3 terms must fit side by side (5 kp <= 256)");
    return go(k_tc_op<IS_K1, 5, true, Cfg, kTyE4M3, CL, TILES>);
  }
  if (nsplit == 1) return go(k_tc_op<IS_K1, 1, false, Cfg, kTyBf16, CL, TILES>);
  CO_CHECK(side, COHERIT_E_SHAPE, "split terms must fit side by side (nsplit * kp <= 256)");
  if (nsplit == 2) return go(k_tc_op<IS_K1, 2, true, Cfg, kTyBf16, CL, TILES>);
  return go(k_tc_op<IS_K1, 3, true, Cfg, kTyBf16, CL, TILES>);
}

// Built forms: single CTAs with one or two tiles, clusters of 2 CTAs with
// one tile each.
template <bool IS_K1, class Cfg>
static int launch_tc_cl(const TcLaunchCfg& cfg, int nsplit, int ty, dim3 grid, cudaStream_t st,
                        const TcParams& p) {
  CO_CHECK((cfg.cluster == 1 || cfg.cluster == 2) && (cfg.tiles == 1 || cfg.tiles == 2) &&
               !(cfg.cluster == 2 && cfg.tiles == 2),
           COHERIT_E_SHAPE, "no operator kernel for %d CTAs per cluster with %d tiles per CTA",
           cfg.cluster, cfg.tiles);
  if (cfg.tiles == 2)
    return launch_tc_cfg<IS_K1, Cfg, 1, 2>(nsplit, ty, cfg.side, grid, cfg.smem, st, p);
  if (cfg.cluster == 2)
    return launch_tc_cfg<IS_K1, Cfg, 2, 1>(nsplit, ty, cfg.side, grid, cfg.smem, st, p);
  return launch_tc_cfg<IS_K1, Cfg, 1, 1>(nsplit, ty, cfg.side, grid, cfg.smem, st, p);
}

// grid.x = row tiles; the launch gives each CTA cfg.tiles of them and rounds
// the CTA count up to whole clusters.
template <bool IS_K1>
static int launch_tc(const TcLaunchCfg& cfg, int nsplit, int ty, dim3 grid, cudaStream_t st,
                     const TcParams& p0) {
  TcParams p = p0;
  p.n_tiles = grid.x;
  const unsigned cl = static_cast<unsigned>(cfg.cluster);
  const unsigned tl = static_cast<unsigned>(cfg.tiles);
  grid.x = (grid.x + tl - 1) / tl;
  grid.x = (grid.x + cl - 1) / cl * cl;
  if (cfg.wide) return launch_tc_cl<IS_K1, CfgWide>(cfg, nsplit, ty, grid, st, p);
  return launch_tc_cl<IS_K1, CfgNarrow>(cfg, nsplit, ty, grid, st, p);
}

// Column-block width when k exceeds what one launch holds (each block
// re-reads the genotypes); k itself otherwise.
static int column_step(int k, int kmax) {
  if (k <= kmax) return k;
  const int nblk = (k + kmax - 1) / kmax;
  return static_cast<int>(round_up((k + nblk - 1) / nblk, 16));
}

static int launch_operator(coherit_geno* h, const OpDesc& d, int kp, int nsplit, uint8_t* ws,
                           cudaStream_t st);

int run_operator(coherit_geno* h, const OpDesc& d, cudaStream_t st) {
  if (d.precision == COHERIT_PREC_AUTO) {
    OpDesc r = d;
    r.precision = resolve_precision(d.precision, d.k);
    if (r.precision == COHERIT_PREC_FP8X5 || d.k <= max_kp_for(h, 3, 2) || d.n_groups > 1)
      return run_operator(h, r, st);
    // Wider than one BF16x3 launch: column blocks, each resolved by width.
    const int step = column_step(d.k, max_kp_for(h, 3, 2));
    for (int c0 = 0; c0 < d.k; c0 += step) {
      OpDesc s = d;
      s.k = std::min(step, d.k - c0);
      s.V = d.V + c0;
      s.out = d.out + c0;
      s.col_start = {0, s.k};
      int rc = run_operator(h, s, st);
      if (rc != COHERIT_OK) return rc;
    }
    return COHERIT_OK;
  }
  if (d.precision == COHERIT_PREC_FP32) return run_operator_fp32(h, d, st);
  CO_CHECK(is_tc_precision(d.precision), COHERIT_E_SHAPE, "unknown precision %d", d.precision);
  const int nsplit = nsplit_of(d.precision);
  const int kmax = max_kp_for(h, nsplit, elem_bytes(d.precision));
  if (d.k > kmax) {
    // Column blocks: each re-reads the genotypes.
    CO_CHECK(d.n_groups == 1, COHERIT_E_SHAPE,
             "batched requests wider than %d columns in one launch are not supported", kmax);
    const int step = column_step(d.k, kmax);
    for (int c0 = 0; c0 < d.k; c0 += step) {
      OpDesc s = d;
      s.k = std::min(step, d.k - c0);
      s.V = d.V + c0;
      s.out = d.out + c0;
      s.col_start = {0, s.k};
      int rc = run_operator(h, s, st);
      if (rc != COHERIT_OK) return rc;
    }
    return COHERIT_OK;
  }
  const int kp = static_cast<int>(round_up(std::max(d.k, 1), 16));
  int rc = ensure_workspace(h, kp, d.precision);
  if (rc != COHERIT_OK) return rc;
  return launch_operator(h, d, kp, nsplit, static_cast<uint8_t*>(h->ws.base), st);
}

int run_operator_in_scratch(coherit_geno* h, const OpDesc& d0, void* scratch, size_t bytes,
                            cudaStream_t st) {
  OpDesc d = d0;
  if (d.precision == COHERIT_PREC_AUTO)
    d.precision = resolve_precision(d.precision, std::min<int32_t>(d.k, kAutoFp8MaxCols + 1));
  CO_CHECK(d.precision != COHERIT_PREC_FP32, COHERIT_E_UNSUPPORTED,
           "the fixed-scratch operator runs the tensor-core precisions only");
  CO_CHECK(is_tc_precision(d.precision), COHERIT_E_SHAPE, "unknown precision %d", d.precision);
  CO_CHECK(d.n_groups == 1, COHERIT_E_SHAPE, "the fixed-scratch operator takes one request");
  const int nsplit = nsplit_of(d.precision);
  const int step = column_step(d.k, max_kp_for(h, nsplit, elem_bytes(d.precision)));
  const int kp = static_cast<int>(round_up(std::max(step, 1), 16));
  const size_t need = ws_layout(h, kp, d.precision).total;
  CO_CHECK(need <= bytes, COHERIT_E_SHAPE,
           "operator needs %zu bytes of scratch for n=%lld, m_pad=%lld, %d columns per launch; "
           "the fixed scratch holds %zu bytes (use coherit_geno_kv)",
           need, static_cast<long long>(h->n), static_cast<long long>(h->m_pad), kp, bytes);
  for (int c0 = 0; c0 < d.k; c0 += step) {
    OpDesc s = d;
    s.k = std::min(step, d.k - c0);
    s.V = d.V + c0;
    s.out = d.out + c0;
    s.col_start = {0, s.k};
    const int kps = static_cast<int>(round_up(s.k, 16));
    int rc = launch_operator(h, s, kps, nsplit, static_cast<uint8_t*>(scratch), st);
    if (rc != COHERIT_OK) return rc;
  }
  return COHERIT_OK;
}

// One launch sequence (prep, K1, K2, corrections) for k <= max_kp_for columns
// with the workspace at `ws` (laid out by ws_layout(h, kp, nsplit)).
static int launch_operator(coherit_geno* h, const OpDesc& d, int kp, int nsplit, uint8_t* ws,
                           cudaStream_t st) {
  const bool f16 = is_scaled(d.precision);  // per-column scales (FP16 or E4M3 terms)
  const int ty = op_type(d.precision);
  const WsLayout L = ws_layout(h, kp, d.precision);
  EpiParams e;
  int rc = fill_epi(h, d, kp, nsplit, e);
  if (rc != COHERIT_OK) return rc;
  auto* vt = reinterpret_cast<__nv_bfloat16*>(ws + L.vt);
  auto* sbuf = reinterpret_cast<__nv_bfloat16*>(ws + L.sbuf);
  auto* cs_part = reinterpret_cast<double*>(ws + L.cs_part);
  auto* cs = reinterpret_cast<float*>(ws + L.cs);
  auto* shift = reinterpret_cast<float*>(ws + L.shift);
  auto* vscale = reinterpret_cast<float*>(ws + L.vscale);
  auto* smax = reinterpret_cast<unsigned*>(ws + L.smax);
  float* mx_part = f16 ? reinterpret_cast<float*>(ws + L.mx_part) : nullptr;
  auto* rbuf = reinterpret_cast<double*>(ws + L.rbuf);
  float* vmiss = h->n_missing > 0 ? reinterpret_cast<float*>(ws + L.vmiss) : nullptr;
  float* sf32 = (h->n_missing > 0 || f16) ? reinterpret_cast<float*>(ws + L.sf32) : nullptr;
  e.cs = cs;
  e.shift = shift;
  e.vscale = vscale;
  e.smax = smax;
  e.vmiss = vmiss;
  e.sbuf = sbuf;
  e.sf32 = sf32;
  e.rbuf = rbuf;
  const int nr = e.stacked ? h->G : 1;
  CO_CUDA(cudaMemsetAsync(rbuf, 0, sizeof(double) * nr * kp, st));
  if (f16) CO_CUDA(cudaMemsetAsync(smax, 0, sizeof(unsigned) * kp, st));
  const TcLaunchCfg cfg = tc_config(h, kp, d.precision);
  const SplitPlan sp =
      split_plan(h, e.stacked != 0, target_ctas_for(h, kp, d.precision), cfg.sb, cfg.tiles);
  float* part = reinterpret_cast<float*>(ws + L.part);
  const unsigned col_blocks = static_cast<unsigned>((kp / 16 + 3) / 4);

  TcParams p;
  memset(&p, 0, sizeof(p));
  p.RB = cfg.RB;
  p.RA = cfg.RA;
  p.RG = cfg.RG;
  p.bslot_bytes = cfg.bslot;
  p.tmem_cols = cfg.tmem_cols;
  p.acc_cols = cfg.acc_cols;
  p.err = h->d_err;
  p.n_chunks = h->n_chunks;
  p.n_panels = h->n_panels;
  p.b_chunk_bytes = static_cast<int64_t>(nsplit) * kp * kPanel * elem_bytes(d.precision);

  if (!d.zxb) {
    // Column means a of V, then V' = V - a split into K1's B tiles and the
    // column sums of V'.
    const int prep_smem = kPanel * (kp + 1) * static_cast<int>(sizeof(float));
    CO_CUDA(cudaFuncSetAttribute(k_prep_v<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 prep_smem));
    CO_CUDA(cudaFuncSetAttribute(k_prep_v<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 prep_smem));
    k_prep_v<false><<<static_cast<unsigned>(h->n_chunks), 256, prep_smem, st>>>(
        d.V, d.ldv, h->n, d.k, kp, nsplit, vt, cs_part, mx_part, e); note_launch();
    k_shift_finish<<<kp, 256, 0, st>>>(cs_part, mx_part, h->n_chunks, kp, shift, vscale, e);
    note_launch();
    k_prep_v<true><<<static_cast<unsigned>(h->n_chunks), 256, prep_smem, st>>>(
        d.V, d.ldv, h->n, d.k, kp, nsplit, vt, cs_part, nullptr, e); note_launch();
    k_colsum_finish<<<kp, 256, 0, st>>>(cs_part, h->n_chunks, kp, cs); note_launch();
    CO_CHECK(vmiss == nullptr || (h->d_csc_off != nullptr && h->d_csc_idx != nullptr),
             COHERIT_E_SHAPE, "missing-genotype lists absent");
    if (vmiss != nullptr)
      k_vmiss<<<static_cast<unsigned>((h->m_pad + 7) / 8), 256, 0, st>>>(
          h->d_csc_off, h->d_csc_idx, h->m_pad, d.V, d.ldv, h->n, d.k, kp, vmiss, e); note_launch();
    CO_CUDA(cudaGetLastError());
    p.geno = h->geno_t;
    p.bsrc = reinterpret_cast<const uint8_t*>(vt);
    p.e = e;
    p.ksplit = sp.k1;
    p.part = sp.k1 > 1 ? part : nullptr;
    p.part_stride = h->m_pad * kp;
    p.part_rows = h->m_pad;
    rc = launch_tc<true>(cfg, nsplit, ty,
                         dim3(static_cast<unsigned>(h->n_ttiles), 1, static_cast<unsigned>(sp.k1)),
                         st, p);
    if (rc != COHERIT_OK) return rc;
    if (sp.k1 > 1) {
      k_k1_finish<<<dim3(static_cast<unsigned>(h->m_pad / 32), col_blocks), dim3(32, 4), 0, st>>>(
          part, sp.k1, p.part_stride, e); note_launch();
      CO_CUDA(cudaGetLastError());
    }
    if (d.xtv) return COHERIT_OK;
  } else {
    // Z b: S = inv_sd * b computed directly.  vscale is never read here.
    CO_CHECK(h->n_missing == 0 || sf32 != nullptr, COHERIT_E_SHAPE, "workspace missing");
    k_prep_s_from_b<<<static_cast<unsigned>((h->m_pad + 127) / 128), 128, 0, st>>>(d.V, d.ldv, e); note_launch();
    CO_CUDA(cudaGetLastError());
  }
  if (f16) {
    // S's column maxima are known once every slot tile is done: FP16 tiles now.
    CO_CHECK(kp <= kMaxSplitCols, COHERIT_E_SHAPE, "scaled forms take at most %d columns",
             kMaxSplitCols);
    k_split_s<<<static_cast<unsigned>((h->m_pad + kSplitThreads - 1) / kSplitThreads),
                kSplitThreads, 0, st>>>(e); note_launch();
    CO_CUDA(cudaGetLastError());
  }
  p.geno = h->geno_s;
  p.bsrc = reinterpret_cast<const uint8_t*>(sbuf);
  p.comp_slot_start = h->d_comp_slot_start;
  p.e = e;
  p.ksplit = sp.k2;
  p.part = sp.k2 > 1 ? part : nullptr;
  p.part_stride = static_cast<int64_t>(nr) * h->n_pad * kp;
  p.part_rows = h->n_pad;
  rc = launch_tc<false>(cfg, nsplit, ty,
                        dim3(static_cast<unsigned>(h->n_stiles), static_cast<unsigned>(nr),
                             static_cast<unsigned>(sp.k2)),
                        st, p);
  if (rc != COHERIT_OK) return rc;
  if (sp.k2 > 1) {
    k_k2_finish<<<dim3(static_cast<unsigned>(h->n_pad / 32), col_blocks, static_cast<unsigned>(nr)),
                  dim3(32, 4), 0, st>>>(part, sp.k2, p.part_stride, h->n_pad, e); note_launch();
    CO_CUDA(cudaGetLastError());
  }
  // Missing-genotype correction: only when the handle holds missing
  // genotypes (and so the CSR lists); the FP32 S buffer also exists for FP16X2.
  if (h->n_missing > 0) {
    CO_CHECK(sf32 != nullptr && h->d_csr_off != nullptr && h->d_csr_idx != nullptr,
             COHERIT_E_SHAPE, "missing-genotype lists or FP32 S buffer absent");
    k_rowcorr<<<static_cast<unsigned>((h->n + 7) / 8), 256, 0, st>>>(h->d_csr_off, h->d_csr_idx,
                                                                      h->n, e); note_launch();
    CO_CUDA(cudaGetLastError());
  }
  return COHERIT_OK;
}

}  // namespace coherit

using namespace coherit;

static int make_single(coherit_geno_t* h, int32_t slot, int32_t k, const float* comp_scale,
                       OpDesc& d) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(k >= 1, COHERIT_E_SHAPE, "right-hand side must have at least one column");
  CO_CHECK(slot >= 0 && slot < static_cast<int32_t>(h->slots.size()) && h->slots[slot].used,
           COHERIT_E_INDEX, "stats slot %d is not initialised", slot);
  d.n_groups = 1;
  d.col_start = {0, k};
  d.slot_of_group = {slot};
  d.comp_scale.assign(h->G, 1.f);
  if (comp_scale != nullptr)
    for (int g = 0; g < h->G; ++g) d.comp_scale[g] = comp_scale[g];
  d.k = k;
  return COHERIT_OK;
}

extern "C" {

int coherit_geno_reserve(coherit_geno_t* h, int32_t k_max, int32_t precision) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  const int kp = static_cast<int>(round_up(std::max(k_max, 1), 16));
  if (precision == COHERIT_PREC_FP32)
    return ensure_ws_bytes(h, static_cast<size_t>(h->m_pad) * kp * sizeof(float));
  if (precision == COHERIT_PREC_AUTO) {
    // Both forms AUTO may pick: E4M3 up to 48 columns, BF16x3 above.
    int rc = coherit_geno_reserve(h, std::min(k_max, kAutoFp8MaxCols), COHERIT_PREC_FP8X5);
    if (rc != COHERIT_OK || k_max <= kAutoFp8MaxCols) return rc;
    return coherit_geno_reserve(h, k_max, COHERIT_PREC_BF16X3);
  }
  CO_CHECK(is_tc_precision(precision), COHERIT_E_SHAPE, "unknown precision %d", precision);
  const int ns = nsplit_of(precision);
  return ensure_workspace(h, std::min(kp, max_kp_for(h, ns, elem_bytes(precision))), precision);
}

int coherit_geno_autotune(coherit_geno_t* h, int32_t k, int32_t precision, int32_t reps,
                          int32_t* choice, float* best_ms, float* default_ms, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(k >= 1 && reps >= 1, COHERIT_E_SHAPE, "autotune needs k >= 1 and reps >= 1");
  const int prec = resolve_precision(precision, k);
  CO_CHECK(is_tc_precision(prec), COHERIT_E_UNSUPPORTED,
           "the autotuner tunes the tensor-core precisions only");
  const int ns = nsplit_of(prec);
  const int kp = static_cast<int>(round_up(k, 16));
  CO_CHECK(kp <= max_kp_for(h, ns, elem_bytes(prec)), COHERIT_E_SHAPE,
           "autotune width %d exceeds one launch (%d columns)", k,
           max_kp_for(h, ns, elem_bytes(prec)));
  CO_CHECK(!h->slots.empty() && h->slots[0].used, COHERIT_E_INDEX, "stats slot 0 is not initialised");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const std::pair<int, int> key{kp, prec};
  h->tuned.erase(key);
  int rc = ensure_workspace(h, kp, prec);
  if (rc != COHERIT_OK) return rc;
  float* buf = nullptr;
  CO_CUDA(cudaMalloc(&buf, sizeof(float) * 2 * h->n * kp));
  CO_CUDA(cudaMemsetAsync(buf, 0, sizeof(float) * h->n * kp, st));
  OpDesc d;
  rc = make_single(h, 0, kp, nullptr, d);
  d.mode = COHERIT_MODE_SUM;
  d.precision = prec;
  d.V = buf;
  d.ldv = kp;
  d.out = buf + h->n * kp;
  d.ldo = kp;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  int nrep = reps;
  auto time_once = [&](float& ms) -> int {
    int r = run_operator(h, d, st);  // warm
    if (r != COHERIT_OK) return r;
    CO_CUDA(cudaEventRecord(e0, st));
    for (int i = 0; i < nrep && r == COHERIT_OK; ++i) r = run_operator(h, d, st);
    if (r != COHERIT_OK) return r;
    CO_CUDA(cudaEventRecord(e1, st));
    CO_CUDA(cudaEventSynchronize(e1));
    CO_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    ms /= static_cast<float>(nrep);
    return COHERIT_OK;
  };
  float t_def = 0.f;
  if (rc == COHERIT_OK && ce == cudaSuccess) rc = time_once(t_def);
  TuneChoice def;
  {
    const TcLaunchCfg c0 = tc_config_policy(h, kp, prec, LaunchReq());
    def.wide = c0.wide ? 1 : 0;
    def.RA = c0.RA;
    def.RB = c0.RB;
    def.RG = c0.RG;
    def.target_mult = kDefaultTargetMult;
    def.cluster = c0.cluster;
    def.tiles = c0.tiles;
    def.ms = t_def;
  }
  std::vector<TuneChoice> timed;
  int tried = 0;
  auto try_choice = [&](TuneChoice c) {
    if (rc != COHERIT_OK || ce != cudaSuccess) return;
    h->tuned[key] = c;
    float ms = 0.f;
    rc = time_once(ms);
    ++tried;
    if (rc == COHERIT_OK) {
      c.ms = ms;
      timed.push_back(c);
    }
  };
  // Candidates: tiles per CTA x stage size x genotype-ring depth (full, or
  // two stages per decoder set where that frees shared memory for another B
  // slot) x A-ring depth x B-ring depth x split-K grid.
  for (int tiles = 1; tiles <= 2; ++tiles) {
    for (int wide = 1; wide >= 0; --wide) {
      LaunchReq rq;
      rq.wide = wide;
      rq.tiles = tiles;
      const TcLaunchCfg full = tc_config_policy(h, kp, prec, rq);
      if ((full.wide ? 1 : 0) != wide || full.tiles != tiles) continue;  // rings do not fit
      const int sets = wide ? CfgWide::SETS : CfgNarrow::SETS;
      const int rgs[2] = {full.RG, 2 * sets};
      for (int ig = 0; ig < 2; ++ig) {
        rq.RG = rgs[ig];
        const TcLaunchCfg fg = tc_config_policy(h, kp, prec, rq);
        if (ig == 1 && (rgs[1] == rgs[0] || fg.RB <= full.RB)) continue;
        const int ra_min = wide ? CfgWide::MIN_RA : CfgNarrow::MIN_RA;
        const int ras[2] = {fg.RA, std::max(ra_min, fg.RA / 2)};
        const int rbs[3] = {fg.RB, std::max(2, fg.RB / 2), 2};
        for (int ia = 0; ia < 2; ++ia) {
          if (ia == 1 && ras[1] == ras[0]) continue;
          for (int ib = 0; ib < 3; ++ib) {
            if ((ib == 1 && rbs[1] == rbs[0]) ||
                (ib == 2 && (rbs[2] == rbs[1] || rbs[2] == rbs[0])))
              continue;
            for (int mult = 2; mult <= kMaxTargetMult; mult *= 2) {
              TuneChoice c;
              c.cluster = 1;
              c.tiles = tiles;
              c.wide = wide;
              c.RG = rgs[ig];
              c.RA = ras[ia];
              c.RB = rbs[ib];
              c.target_mult = mult;
              try_choice(c);
            }
          }
        }
      }
    }
  }
  // Clusters of 2 CTAs sharing every B tile, on the best one-tile rings.
  {
    TuneChoice b1 = def;
    for (const TuneChoice& c : timed)
      if (c.tiles == 1 && c.ms < b1.ms) b1 = c;
    for (int mult = 2; mult <= kMaxTargetMult; mult *= 2) {
      TuneChoice c = b1;
      c.cluster = 2;
      c.tiles = 1;
      c.target_mult = mult;
      try_choice(c);
    }
  }
  // One timed application is noisy (clock and power state): re-time the
  // fastest three and the fixed policy with three times the repetitions
  // and keep the fastest.
  TuneChoice best = def;
  if (rc == COHERIT_OK && ce == cudaSuccess) {
    std::sort(timed.begin(), timed.end(),
              [](const TuneChoice& x, const TuneChoice& y) { return x.ms < y.ms; });
    if (timed.size() > 3) timed.resize(3);
    timed.push_back(def);
    nrep = 3 * reps;
    best.ms = 3.4e38f;
    for (TuneChoice c : timed) {
      if (rc != COHERIT_OK) break;
      h->tuned[key] = c;
      float ms = 0.f;
      rc = time_once(ms);
      if (rc == COHERIT_OK && ms < best.ms) {
        best = c;
        best.ms = ms;
      }
      if (c.wide == def.wide && c.RA == def.RA && c.RB == def.RB && c.RG == def.RG &&
          c.target_mult == def.target_mult && c.cluster == def.cluster && c.tiles == def.tiles)
        t_def = ms;
    }
  }
  h->tuned[key] = best;
  if (rc == COHERIT_OK && ce == cudaSuccess) {
    int herr = 0;
    ce = cudaMemcpy(&herr, h->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && herr != 0) {
      set_error("operator kernel reported error %d while tuning", herr);
      rc = COHERIT_E_CUDA;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(buf);
  if (rc != COHERIT_OK) {
    h->tuned.erase(key);
    return rc;
  }
  if (ce != cudaSuccess) return cuda_status(ce, "autotune");
  if (choice) {
    choice[0] = best.wide;
    choice[1] = best.RA;
    choice[2] = best.RB;
    choice[3] = best.target_mult;
    choice[4] = tried;
    choice[5] = best.cluster;
    choice[6] = best.RG;
    choice[7] = best.tiles;
  }
  if (best_ms) *best_ms = best.ms;
  if (default_ms) *default_ms = t_def;
  return COHERIT_OK;
}

int coherit_geno_set_launch(coherit_geno_t* h, int32_t k, int32_t precision,
                            const int32_t* cfg) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(k >= 1, COHERIT_E_SHAPE, "width must be >= 1");
  const int prec = resolve_precision(precision, k);
  CO_CHECK(is_tc_precision(prec), COHERIT_E_UNSUPPORTED,
           "launch configurations exist for the tensor-core precisions only");
  const std::pair<int, int> key{static_cast<int>(round_up(k, 16)), prec};
  if (cfg == nullptr) {
    h->tuned.erase(key);
    return COHERIT_OK;
  }
  CO_CHECK(cfg[0] == 0 || cfg[0] == 1, COHERIT_E_SHAPE, "stage form must be 0 or 1");
  CO_CHECK(cfg[1] >= 0 && cfg[1] <= kMaxRA && cfg[2] >= 0 && cfg[2] <= kMaxRB, COHERIT_E_SHAPE,
           "ring depths must lie in [0, %d] and [0, %d] (0 = largest that fits)", kMaxRA,
           kMaxRB);
  CO_CHECK(cfg[3] == 2 || cfg[3] == 4 || cfg[3] == 8, COHERIT_E_SHAPE,
           "grid multiple must be 2, 4 or 8");
  CO_CHECK(cfg[5] == 1 || cfg[5] == 2, COHERIT_E_SHAPE, "CTAs per cluster must be 1 or 2");
  CO_CHECK(cfg[6] >= 0 && cfg[6] <= CfgNarrow::RG, COHERIT_E_SHAPE,
           "genotype ring depth must lie in [0, %d] (0 = full)", CfgNarrow::RG);
  CO_CHECK(cfg[7] == 1 || cfg[7] == 2, COHERIT_E_SHAPE, "tiles per CTA must be 1 or 2");
  CO_CHECK(!(cfg[5] == 2 && cfg[7] == 2), COHERIT_E_SHAPE,
           "clusters of 2 CTAs run one tile per CTA");
  TuneChoice c;
  c.RG = cfg[6];
  c.tiles = cfg[7];
  c.wide = cfg[0];
  c.RA = cfg[1];
  c.RB = cfg[2];
  c.target_mult = cfg[3];
  c.cluster = cfg[5];
  h->tuned[key] = c;
  return COHERIT_OK;
}

int coherit_geno_kv(coherit_geno_t* h, int32_t slot, int32_t mode, int32_t precision,
                    const float* V, int64_t ldv, int32_t k, const float* comp_scale,
                    int32_t use_theta_e, float theta_e, const float* snp_weight, float* out,
                    int64_t ldo, void* stream) {
  OpDesc d;
  int rc = make_single(h, slot, k, comp_scale, d);
  if (rc != COHERIT_OK) return rc;
  CO_CHECK(mode == COHERIT_MODE_SUM || mode == COHERIT_MODE_STACKED, COHERIT_E_SHAPE,
           "unknown operator mode %d", mode);
  CO_CHECK(ldv >= k && ldo >= k, COHERIT_E_SHAPE, "row strides must be >= k");
  CO_CHECK(V != nullptr && out != nullptr, COHERIT_E_SHAPE, "V and out are required");
  d.mode = mode;
  d.precision = precision;
  if (use_theta_e && mode == COHERIT_MODE_SUM) d.theta_e = {theta_e};
  d.snp_weight = snp_weight;
  d.V = V;
  d.ldv = ldv;
  d.out = out;
  d.ldo = ldo;
  return run_operator(h, d, static_cast<cudaStream_t>(stream));
}

int coherit_geno_kv_batched(coherit_geno_t* h, int32_t n_requests, const int32_t* col_start,
                            const int32_t* slots, int32_t precision, const float* V, int64_t ldv,
                            int32_t k, const float* comp_scale, const float* theta_e, float* out,
                            int64_t ldo, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(n_requests >= 1, COHERIT_E_SHAPE, "need at least one request");
  CO_CHECK(col_start[0] == 0 && col_start[n_requests] == k, COHERIT_E_SHAPE,
           "column groups must cover [0, k)");
  OpDesc d;
  d.n_groups = n_requests;
  d.col_start.assign(col_start, col_start + n_requests + 1);
  for (int r = 0; r < n_requests; ++r)
    CO_CHECK(col_start[r + 1] > col_start[r], COHERIT_E_SHAPE, "request %d has no columns", r);
  d.slot_of_group.assign(slots, slots + n_requests);
  d.comp_scale.assign(comp_scale, comp_scale + static_cast<size_t>(n_requests) * h->G);
  if (theta_e != nullptr) d.theta_e.assign(theta_e, theta_e + n_requests);
  d.precision = precision;
  d.V = V;
  d.ldv = ldv;
  d.k = k;
  d.out = out;
  d.ldo = ldo;
  return run_operator(h, d, static_cast<cudaStream_t>(stream));
}

int coherit_geno_xtv(coherit_geno_t* h, int32_t slot, int32_t precision, const float* V,
                     int64_t ldv, int32_t k, const float* comp_scale, float* out, int64_t ldo,
                     void* stream) {
  OpDesc d;
  int rc = make_single(h, slot, k, comp_scale, d);
  if (rc != COHERIT_OK) return rc;
  d.xtv = true;
  d.precision = precision;
  d.V = V;
  d.ldv = ldv;
  d.out = out;
  d.ldo = ldo;
  return run_operator(h, d, static_cast<cudaStream_t>(stream));
}

int coherit_geno_zxb(coherit_geno_t* h, int32_t slot, int32_t precision, const float* b,
                     int64_t ldb, int32_t C, float* out, int64_t ldo, void* stream) {
  OpDesc d;
  int rc = make_single(h, slot, C, nullptr, d);
  if (rc != COHERIT_OK) return rc;
  d.zxb = true;
  d.precision = precision;
  d.V = b;
  d.ldv = ldb;
  d.out = out;
  d.ldo = ldo;
  return run_operator(h, d, static_cast<cudaStream_t>(stream));
}

}  // extern "C"

// Kernel parameters stay within the classic 4 KB limit.
static_assert(sizeof(coherit::TcParams) <= 4000, "operator kernel parameters exceed 4 KB");
