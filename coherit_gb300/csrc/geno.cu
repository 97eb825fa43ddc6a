// geno.cu -- resident genotype matrix: creation (from the reference's packed
// cache or from the synthetic generator), the two HBM layouts, per-SNP
// statistics, missing-genotype lists, exact diagonal, and the C entry points
// that manage the handle.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <algorithm>
#include <cmath>

#include "coherit_internal.cuh"

namespace coherit {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int cuda_status(cudaError_t e, const char* what) {
  set_error("CUDA error %d (%s) in %s", static_cast<int>(e), cudaGetErrorString(e), what);
  if (e == cudaErrorMemoryAllocation) return COHERIT_E_OOM;
  return COHERIT_E_CUDA;
}

// ------------------------------------------------------------ layout kernels

// copy S from the reference layout: one thread per (sample row, panel).
__global__ void k_build_s_from_ref(uint8_t* __restrict__ geno_s, int64_t n, int64_t n_pad,
                                   int64_t n_panels, const uint8_t* __restrict__ packed,
                                   const int64_t* __restrict__ call_off,
                                   const int32_t* __restrict__ call_pw,
                                   const int32_t* __restrict__ snp_call,
                                   const int32_t* __restrict__ snp_col,
                                   const int32_t* __restrict__ snp_of_slot) {
  const int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (idx >= n_pad * n_panels) return;
  const int64_t p = idx % n_panels;
  const int64_t i = idx / n_panels;
  uint32_t w[4] = {0u, 0u, 0u, 0u};
  if (i < n) {
    for (int e = 0; e < kPanel; ++e) {
      const int32_t s = snp_of_slot[p * kPanel + e];
      if (s < 0) continue;
      const int32_t c = snp_call[s];
      const int32_t col = snp_col[s];
      const uint8_t byte = packed[call_off[c] + i * static_cast<int64_t>(call_pw[c]) + (col >> 2)];
      const uint32_t code = (byte >> (2 * (col & 3))) & 3u;
      w[row_word(e)] |= code << row_shift(e);
    }
  }
  const int64_t st = i / kTile;
  uint4* dst = reinterpret_cast<uint4*>(geno_s + ((st * n_panels + p) * kTile + (i % kTile)) *
                                                     kRowBytes);
  *dst = make_uint4(w[0], w[1], w[2], w[3]);
}

// copy S from SNP-major PLINK BED records of cache SNPs [s_lo, s_hi) (one
// record of `bps` bytes per SNP, sample k at bits 2*(k%4) of byte k/4; BED
// codes 0,1,2,3 -> allele count 2, missing, 1, 0 as the reference's BED
// transcode, geno_stream.py:709-745).  keep: source sample of each row
// (nullptr = identity).  Rows of panels [p_lo, p_hi) are OR-ed into copy S
// (zeroed beforehand), so a panel may be filled by consecutive chunks.
__global__ void k_build_s_from_bed(uint8_t* __restrict__ geno_s, int64_t n, int64_t n_pad,
                                   int64_t n_panels, const uint8_t* __restrict__ bed, int64_t bps,
                                   int64_t s_lo, int64_t s_hi, const int32_t* __restrict__ keep,
                                   const int32_t* __restrict__ snp_of_slot, int64_t p_lo,
                                   int64_t p_hi) {
  const int64_t np = p_hi - p_lo;
  const int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (idx >= n * np) return;
  // Consecutive threads take consecutive samples of one panel, so a warp
  // reads 8 neighbouring bytes of each SNP record.
  const int64_t i = idx % n;
  const int64_t p = p_lo + idx / n;
  const int64_t ks = keep ? keep[i] : i;
  const int64_t byte_off = ks >> 2;
  const int shift = static_cast<int>(2 * (ks & 3));
  uint32_t w[4] = {0u, 0u, 0u, 0u};
  for (int e = 0; e < kPanel; ++e) {
    const int32_t snp = snp_of_slot[p * kPanel + e];
    if (snp < s_lo || snp >= s_hi) continue;
    const uint32_t b = (bed[(snp - s_lo) * bps + byte_off] >> shift) & 3u;
    const uint32_t code = (0x1Eu >> (2 * b)) & 3u;  // BED 0,1,2,3 -> 2, 3 (missing), 1, 0
    w[row_word(e)] |= code << row_shift(e);
  }
  const int64_t st = i / kTile;
  uint4* dst = reinterpret_cast<uint4*>(geno_s + ((st * n_panels + p) * kTile + (i % kTile)) *
                                                     kRowBytes);
  const uint4 old = *dst;
  *dst = make_uint4(old.x | w[0], old.y | w[1], old.z | w[2], old.w | w[3]);
}

// Block-LD generator (genotypes with linkage disequilibrium, for the
// 8-component benchmark workload).  SNPs come in blocks of `block`; every
// sample carries two latent haplotype chains per block,
//   x_0 = e_0,  x_p = rho_b x_{p-1} + s_b e_p   (FP32, each operation rounded),
// with e drawn from a 4096-entry table of standard-normal quantiles indexed
// by the top 12 bits of a counter-based hash of (seed, SNP, sample,
// haplotype); allele = [x_p < thr_j], genotype = sum of the two alleles, so
// every allele is Bernoulli(Phi(thr_j)) and neighbouring SNPs share rho_b.
// The tables (thr, rho, s, quantiles) come from the host, where a numpy
// twin of the same arithmetic reproduces every code.  One thread per (4
// consecutive samples, LD block) writes SNP-major PLINK BED records (byte q
// of the record of SNP j holds samples 4q..4q+3; count 2, 1, 0 -> BED code
// 0, 2, 3) at record record_of_snp[j] (identity when null).
__global__ void __launch_bounds__(256) k_ldblock_records(
    uint8_t* __restrict__ out, int64_t n_rows, int64_t bps, int64_t m, int32_t block,
    uint64_t seed, const float* __restrict__ thr, const float* __restrict__ rho,
    const float* __restrict__ sfac, const float* __restrict__ qtab,
    const int64_t* __restrict__ record_of_snp) {
  __shared__ float q[4096];
  for (int t = threadIdx.x; t < 4096; t += blockDim.x) q[t] = qtab[t];
  __syncthreads();
  const int64_t nb = (m + block - 1) / block;
  const int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (idx >= bps * nb) return;
  const int64_t qg = idx % bps;
  const int64_t b = idx / bps;
  const float r = rho[b], sf = sfac[b];
  float x[8];
  const int64_t j0 = b * block, j1 = min(m, j0 + static_cast<int64_t>(block));
  for (int64_t j = j0; j < j1; ++j) {
    const uint64_t ks = synth_snp_key(seed, j);
    const float tj = thr[j];
    uint32_t byte = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int64_t i = qg * 4 + t;
      uint32_t cnt = 0;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const uint64_t hh =
            splitmix64(ks ^ (static_cast<uint64_t>(2 * i + a) * 0x9E3779B97F4A7C15ull));
        const float e = q[hh >> 52];
        x[2 * t + a] = (j == j0) ? e : __fadd_rn(__fmul_rn(r, x[2 * t + a]), __fmul_rn(sf, e));
        cnt += x[2 * t + a] < tj ? 1u : 0u;
      }
      const uint32_t bed = cnt == 2 ? 0u : (cnt == 1 ? 2u : 3u);
      if (i < n_rows) byte |= bed << (2 * t);
    }
    const int64_t rec = record_of_snp ? record_of_snp[j] : j;
    out[rec * bps + qg] = static_cast<uint8_t>(byte);
  }
}

// copy S from the synthetic generator.
__global__ void k_build_s_synth(uint8_t* __restrict__ geno_s, int64_t n, int64_t n_pad,
                                int64_t n_panels, const int32_t* __restrict__ snp_of_slot,
                                uint64_t seed, uint32_t miss_q24) {
  const int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (idx >= n_pad * n_panels) return;
  const int64_t p = idx % n_panels;
  const int64_t i = idx / n_panels;
  uint32_t w[4] = {0u, 0u, 0u, 0u};
  if (i < n) {
    for (int e = 0; e < kPanel; ++e) {
      const int32_t s = snp_of_slot[p * kPanel + e];
      if (s < 0) continue;
      const uint32_t code = synth_code(seed, s, i, synth_maf_q24(seed, s), miss_q24);
      w[row_word(e)] |= code << row_shift(e);
    }
  }
  const int64_t st = i / kTile;
  uint4* dst = reinterpret_cast<uint4*>(geno_s + ((st * n_panels + p) * kTile + (i % kTile)) *
                                                     kRowBytes);
  *dst = make_uint4(w[0], w[1], w[2], w[3]);
}

// copy T from copy S: one CTA (128 threads) per T block (slot tile tt,
// sample chunk q).  The 64 sample rows x 2 panels of copy S are staged in
// shared memory and every thread assembles the 16-byte row of one slot.
__global__ void __launch_bounds__(128) k_build_t_from_s(uint8_t* __restrict__ geno_t,
                                                        const uint8_t* __restrict__ geno_s,
                                                        int64_t n_panels, int64_t n_chunks) {
  __shared__ uint32_t rows[2][kPanel][4];
  const int64_t tt = blockIdx.y;
  const int64_t q = blockIdx.x;
  const int tid = threadIdx.x;
  const int64_t st = (q * kPanel) / kTile;
  const int row0 = static_cast<int>((q * kPanel) % kTile);
  {
    const int panel = tid / kPanel;
    const int r = tid % kPanel;
    const uint4 v = *reinterpret_cast<const uint4*>(
        geno_s + ((st * n_panels + 2 * tt + panel) * kTile + row0 + r) * kRowBytes);
    rows[panel][r][0] = v.x;
    rows[panel][r][1] = v.y;
    rows[panel][r][2] = v.z;
    rows[panel][r][3] = v.w;
  }
  __syncthreads();
  const int panel = tid / kPanel;
  const int e = tid % kPanel;
  const int we = row_word(e), se = row_shift(e);
  uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll 8
  for (int r = 0; r < kPanel; ++r) {
    const uint32_t code = (rows[panel][r][we] >> se) & 3u;
    w[row_word(r)] |= code << row_shift(r);
  }
  uint4* dst = reinterpret_cast<uint4*>(geno_t + ((tt * n_chunks + q) * kTile + tid) * kRowBytes);
  *dst = make_uint4(w[0], w[1], w[2], w[3]);
}

// Reference-layout bytes of SNP (cache) range [s0, s0+width) for all samples.
__global__ void k_read_packed(uint8_t* __restrict__ out, const uint8_t* __restrict__ geno_s,
                              int64_t n, int64_t n_panels, const int64_t* __restrict__ slot_of_snp,
                              int64_t s0, int32_t width) {
  const int32_t pw = (width + 3) / 4;
  const int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (idx >= n * pw) return;
  const int64_t i = idx / pw;
  const int32_t b = static_cast<int32_t>(idx % pw);
  const int64_t st = i / kTile;
  uint32_t byte = 0;
  for (int t = 0; t < 4; ++t) {
    const int32_t col = 4 * b + t;
    if (col >= width) break;
    const int64_t slot = slot_of_snp[s0 + col];
    const int64_t p = slot / kPanel;
    const int e = static_cast<int>(slot % kPanel);
    const uint32_t* row = reinterpret_cast<const uint32_t*>(
        geno_s + ((st * n_panels + p) * kTile + (i % kTile)) * kRowBytes);
    const uint32_t code = (row[row_word(e)] >> row_shift(e)) & 3u;
    byte |= code << (2 * t);
  }
  out[idx] = static_cast<uint8_t>(byte);
}

// Standardised genotype columns: out[i, c] = (g - mean) * inv_sd of SNP
// snp_idx[c] (cache order) for sample i, 0 for a missing genotype (mean
// imputation), in FP32 with the reference's operation order
// (geno_stream.py:2498-2501).  Threads of a warp take consecutive columns so
// the writes of a row are coalesced.  An index outside [0, m) yields NaN.
__global__ void k_extract_std(float* __restrict__ out, int64_t ldo, const int64_t* __restrict__ snp_idx,
                              int32_t count, const uint8_t* __restrict__ geno_t, int64_t n,
                              int64_t m, int64_t n_chunks, const int64_t* __restrict__ slot_of_snp,
                              const float* __restrict__ mean, const float* __restrict__ inv) {
  const int32_t c = static_cast<int32_t>(blockIdx.x) * 32 + threadIdx.x;
  if (c >= count) return;
  const int64_t snp = snp_idx[c];
  const bool valid = snp >= 0 && snp < m;
  const int64_t slot = valid ? slot_of_snp[snp] : 0;
  const float mu = mean[slot];
  const float iv = inv[slot];
  const uint8_t* tile = geno_t + (slot / kTile) * n_chunks * kBlockBytes + (slot % kTile) * kRowBytes;
  for (int64_t i = static_cast<int64_t>(blockIdx.y) * blockDim.y + threadIdx.y; i < n;
       i += static_cast<int64_t>(gridDim.y) * blockDim.y) {
    const uint32_t* row = reinterpret_cast<const uint32_t*>(tile + (i / kPanel) * kBlockBytes);
    const int e = static_cast<int>(i % kPanel);
    const uint32_t code = (row[row_word(e)] >> row_shift(e)) & 3u;
    float z = code == 3u ? 0.f : __fmul_rn(__fsub_rn(static_cast<float>(code), mu), iv);
    if (!valid) z = __int_as_float(0x7fc00000);
    out[i * ldo + c] = z;
  }
}

// ------------------------------------------------------------ statistics

__device__ __forceinline__ void count_codes(uint32_t w, uint32_t mask, int& n1, int& n2,
                                            int& n3) {
  const uint32_t lo = w & 0x55555555u;
  const uint32_t hi = (w >> 1) & 0x55555555u;
  const uint32_t m = mask & 0x55555555u;
  n1 += __popc(lo & ~hi & m);
  n2 += __popc(hi & ~lo & m);
  n3 += __popc(lo & hi & m);
}

// Per-slot genotype counts over the samples of a slot mask (copy T rows).
__global__ void k_slot_counts(const uint8_t* __restrict__ geno_t, int64_t m_pad,
                              int64_t n_chunks, const uint32_t* __restrict__ tmask,
                              int64_t* __restrict__ n1o, int64_t* __restrict__ n2o,
                              int64_t* __restrict__ n3o) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j >= m_pad) return;
  const int64_t tt = j / kTile;
  const int row = static_cast<int>(j % kTile);
  int64_t a1 = 0, a2 = 0, a3 = 0;
  for (int64_t q = 0; q < n_chunks; ++q) {
    const uint4 v = *reinterpret_cast<const uint4*>(
        geno_t + ((tt * n_chunks + q) * kTile + row) * kRowBytes);
    uint4 mk = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
    if (tmask != nullptr) mk = reinterpret_cast<const uint4*>(tmask)[q];
    int n1 = 0, n2 = 0, n3 = 0;
    count_codes(v.x, mk.x, n1, n2, n3);
    count_codes(v.y, mk.y, n1, n2, n3);
    count_codes(v.z, mk.z, n1, n2, n3);
    count_codes(v.w, mk.w, n1, n2, n3);
    a1 += n1;
    a2 += n2;
    a3 += n3;
  }
  n1o[j] = a1;
  n2o[j] = a2;
  n3o[j] = a3;
}

// Sums of diff per slot: dseg[z, j] = s1_jz - cnt_jz mu_j over segment z
// (chunks [64 z, 64 z + 64)) and dsum[j] = s1_j - cnt_j mu_j over all the
// slot's samples, each in FP64 from integer counts, stored in FP32.
// nseg[z] = samples of the slot in segment z.
__global__ void k_slot_seg_dsum(const uint8_t* __restrict__ geno_t, int64_t m_pad,
                                int64_t n_chunks, const uint32_t* __restrict__ tmask,
                                const float* __restrict__ mean, const float* __restrict__ nseg,
                                const int32_t* __restrict__ snp_of_slot, int n_seg,
                                float* __restrict__ dseg, float* __restrict__ dsum) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j >= m_pad) return;
  const int64_t tt = j / kTile;
  const int row = static_cast<int>(j % kTile);
  const bool pad = snp_of_slot[j] < 0;
  const double mu = static_cast<double>(mean[j]);
  double s1_all = 0.0, cnt_all = 0.0;
  for (int z = 0; z < n_seg; ++z) {
    int n1 = 0, n2 = 0, n3 = 0;
    const int64_t q1 = min(n_chunks, static_cast<int64_t>(z + 1) * kSegChunks);
    for (int64_t q = static_cast<int64_t>(z) * kSegChunks; q < q1; ++q) {
      const uint4 v = *reinterpret_cast<const uint4*>(
          geno_t + ((tt * n_chunks + q) * kTile + row) * kRowBytes);
      uint4 mk = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
      if (tmask != nullptr) mk = reinterpret_cast<const uint4*>(tmask)[q];
      count_codes(v.x, mk.x, n1, n2, n3);
      count_codes(v.y, mk.y, n1, n2, n3);
      count_codes(v.z, mk.z, n1, n2, n3);
      count_codes(v.w, mk.w, n1, n2, n3);
    }
    const double cnt = static_cast<double>(nseg[z]) - static_cast<double>(n3);
    const double s1 = static_cast<double>(n1 + 2 * n2);
    dseg[static_cast<int64_t>(z) * m_pad + j] = pad ? 0.f : static_cast<float>(s1 - cnt * mu);
    s1_all += s1;
    cnt_all += cnt;
  }
  dsum[j] = pad ? 0.f : static_cast<float>(s1_all - cnt_all * mu);
}

// Reference FP32 standardisation of every slot (padding slots get 0, 0).
__global__ void k_slot_stats(int64_t m_pad, int64_t n_sub, const int64_t* __restrict__ n1,
                             const int64_t* __restrict__ n2, const int64_t* __restrict__ n3,
                             const int32_t* __restrict__ snp_of_slot, float* __restrict__ mean,
                             float* __restrict__ inv) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j >= m_pad) return;
  if (snp_of_slot[j] < 0) {
    mean[j] = 0.f;
    inv[j] = 0.f;
    return;
  }
  ref_fp32_standardize(n_sub, n1[j], n2[j], n3[j], mean[j], inv[j]);
}

// Missing-genotype counts per sample (copy S rows).
__global__ void k_sample_missing_counts(const uint8_t* __restrict__ geno_s, int64_t n_pad,
                                        int64_t n_panels, int64_t* __restrict__ cnt) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n_pad) return;
  const int64_t st = i / kTile;
  int64_t a = 0;
  for (int64_t p = 0; p < n_panels; ++p) {
    const uint4 v = *reinterpret_cast<const uint4*>(
        geno_s + ((st * n_panels + p) * kTile + (i % kTile)) * kRowBytes);
    const uint32_t ws[4] = {v.x, v.y, v.z, v.w};
    for (int t = 0; t < 4; ++t) a += __popc(ws[t] & (ws[t] >> 1) & 0x55555555u);
  }
  cnt[i] = a;
}

__global__ void k_fill_csc(const uint8_t* __restrict__ geno_t, int64_t m_pad, int64_t n_chunks,
                           const int64_t* __restrict__ off, int32_t* __restrict__ idx) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j >= m_pad) return;
  const int64_t tt = j / kTile;
  const int row = static_cast<int>(j % kTile);
  int64_t pos = off[j];
  const int64_t end = off[j + 1];
  for (int64_t q = 0; q < n_chunks && pos < end; ++q) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(
        geno_t + ((tt * n_chunks + q) * kTile + row) * kRowBytes);
    for (int e = 0; e < kPanel; ++e) {
      if (((w[row_word(e)] >> row_shift(e)) & 3u) == 3u && pos < end) {
        idx[pos++] = static_cast<int32_t>(q * kPanel + e);
      }
    }
  }
}

__global__ void k_fill_csr(const uint8_t* __restrict__ geno_s, int64_t n_pad, int64_t n_panels,
                           const int64_t* __restrict__ off, int32_t* __restrict__ idx) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n_pad) return;
  const int64_t st = i / kTile;
  int64_t pos = off[i];
  const int64_t end = off[i + 1];
  for (int64_t p = 0; p < n_panels && pos < end; ++p) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(
        geno_s + ((st * n_panels + p) * kTile + (i % kTile)) * kRowBytes);
    for (int e = 0; e < kPanel; ++e) {
      if (((w[row_word(e)] >> row_shift(e)) & 3u) == 3u && pos < end) {
        idx[pos++] = static_cast<int32_t>(p * kPanel + e);
      }
    }
  }
}

// Exact diagonal: sum_j z_ij^2 in FP64 (geno_stream.py:929-955).
__global__ void k_exact_diag(const uint8_t* __restrict__ geno_s, int64_t n, int64_t n_panels,
                             const float* __restrict__ mean, const float* __restrict__ inv,
                             const uint8_t* __restrict__ row_mask, double inv_eff,
                             float* __restrict__ out) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  if (row_mask != nullptr && row_mask[i] == 0) {
    out[i] = 0.f;
    return;
  }
  const int64_t st = i / kTile;
  double total = 0.0;
  for (int64_t p = 0; p < n_panels; ++p) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(
        geno_s + ((st * n_panels + p) * kTile + (i % kTile)) * kRowBytes);
    const uint32_t ws[4] = {w[0], w[1], w[2], w[3]};
    for (int e = 0; e < kPanel; ++e) {
      const uint32_t code = (ws[row_word(e)] >> row_shift(e)) & 3u;
      const int64_t j = p * kPanel + e;
      const double iv = static_cast<double>(inv[j]);
      if (code == 3u || iv == 0.0) continue;
      const double z = (static_cast<double>(code) - static_cast<double>(mean[j])) * iv;
      total += z * z;
    }
  }
  out[i] = static_cast<float>(total * inv_eff);
}

// Sample mask in copy-T row order: 2 bits per sample (both set = keep).
__global__ void k_build_tmask(const uint8_t* __restrict__ row_mask, int64_t n, int64_t n_chunks,
                              uint32_t* __restrict__ tmask) {
  const int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (q >= n_chunks) return;
  uint32_t w[4] = {0u, 0u, 0u, 0u};
  for (int e = 0; e < kPanel; ++e) {
    const int64_t i = q * kPanel + e;
    if (i < n && row_mask[i] != 0) w[row_word(e)] |= 3u << row_shift(e);
  }
  for (int t = 0; t < 4; ++t) tmask[4 * q + t] = w[t];
}

static inline unsigned grid_of(int64_t work, int threads) {
  return static_cast<unsigned>((work + threads - 1) / threads);
}

int build_layout_from_ref(coherit_geno* h, const uint8_t* d_packed, const int64_t* d_call_off,
                          const int32_t* d_call_pw, const int32_t* d_snp_call,
                          const int32_t* d_snp_col, cudaStream_t st) {
  const int64_t work = h->n_pad * h->n_panels;
  if (work > 0)
    k_build_s_from_ref<<<grid_of(work, 256), 256, 0, st>>>(
        h->geno_s, h->n, h->n_pad, h->n_panels, d_packed, d_call_off, d_call_pw, d_snp_call,
        d_snp_col, h->d_snp_of_slot); note_launch();
  CO_CUDA(cudaGetLastError());
  return build_copy_t(h, st);
}

// copy S from a host PLINK BED file (bytes after the 3-byte header), uploaded
// and transcoded in chunks of whole SNP records; then copy T.
int build_layout_from_bed(coherit_geno* h, const uint8_t* bed_body, int64_t bps,
                          const int32_t* d_keep, const std::vector<int32_t>& slot_of_snp_host,
                          cudaStream_t st) {
  CO_CUDA(cudaMemsetAsync(h->geno_s, 0, static_cast<size_t>(h->n_pad) * h->m_pad / 4, st));
  // Device staging per chunk: COHERIT_BED_CHUNK_BYTES (default 256 MB) of
  // whole SNP records.
  int64_t chunk_bytes = int64_t(256) << 20;
  if (const char* env = getenv("COHERIT_BED_CHUNK_BYTES")) {
    const long long v = atoll(env);
    if (v > 0) chunk_bytes = v;
  }
  const int64_t chunk = std::max<int64_t>(1, chunk_bytes / std::max<int64_t>(bps, 1));
  uint8_t* d_chunk = nullptr;
  CO_CUDA(cudaMalloc(&d_chunk, static_cast<size_t>(std::min<int64_t>(chunk, h->m)) * bps));
  cudaError_t e = cudaSuccess;
  for (int64_t s_lo = 0; s_lo < h->m && e == cudaSuccess; s_lo += chunk) {
    const int64_t s_hi = std::min<int64_t>(s_lo + chunk, h->m);
    e = cudaMemcpyAsync(d_chunk, bed_body + s_lo * bps, static_cast<size_t>(s_hi - s_lo) * bps,
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) break;
    const int64_t p_lo = slot_of_snp_host[s_lo] / kPanel;
    const int64_t p_hi = slot_of_snp_host[s_hi - 1] / kPanel + 1;
    const int64_t work = h->n * (p_hi - p_lo);
    k_build_s_from_bed<<<grid_of(work, 256), 256, 0, st>>>(
        h->geno_s, h->n, h->n_pad, h->n_panels, d_chunk, bps, s_lo, s_hi, d_keep,
        h->d_snp_of_slot, p_lo, p_hi); note_launch();
    e = cudaGetLastError();
  }
  // The chunk buffer is reused by queued work until the stream drains.
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_chunk);
  if (e != cudaSuccess) return cuda_status(e, "BED transcode");
  return build_copy_t(h, st);
}

int build_layout_synthetic(coherit_geno* h, uint64_t seed, uint32_t miss_q24, cudaStream_t st) {
  const int64_t work = h->n_pad * h->n_panels;
  if (work > 0)
    k_build_s_synth<<<grid_of(work, 256), 256, 0, st>>>(h->geno_s, h->n, h->n_pad, h->n_panels,
                                                        h->d_snp_of_slot, seed, miss_q24); note_launch();
  CO_CUDA(cudaGetLastError());
  return build_copy_t(h, st);
}

int build_copy_t(coherit_geno* h, cudaStream_t st) {
  if (h->n_ttiles > 0 && h->n_chunks > 0) {
    dim3 grid(static_cast<unsigned>(h->n_chunks), static_cast<unsigned>(h->n_ttiles));
    k_build_t_from_s<<<grid, 128, 0, st>>>(h->geno_t, h->geno_s, h->n_panels, h->n_chunks); note_launch();
  }
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

static int exclusive_scan_host(const std::vector<int64_t>& counts, std::vector<int64_t>& off) {
  off.assign(counts.size() + 1, 0);
  for (size_t i = 0; i < counts.size(); ++i) off[i + 1] = off[i] + counts[i];
  return COHERIT_OK;
}

int build_missing_lists(coherit_geno* h, cudaStream_t st) {
  int64_t *d_n1 = nullptr, *d_n2 = nullptr, *d_n3 = nullptr, *d_sc = nullptr;
  CO_CUDA(cudaMalloc(&d_n1, sizeof(int64_t) * h->m_pad * 3));
  d_n2 = d_n1 + h->m_pad;
  d_n3 = d_n2 + h->m_pad;
  k_slot_counts<<<grid_of(h->m_pad, 128), 128, 0, st>>>(h->geno_t, h->m_pad, h->n_chunks, nullptr,
                                                        d_n1, d_n2, d_n3); note_launch();
  std::vector<int64_t> slot_miss(h->m_pad);
  cudaError_t e = cudaMemcpyAsync(slot_miss.data(), d_n3, sizeof(int64_t) * h->m_pad,
                                  cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_n1);
  if (e != cudaSuccess) return cuda_status(e, "missing counts");
  int64_t total = 0;
  for (int64_t v : slot_miss) total += v;
  h->n_missing = total;
  if (total == 0) return COHERIT_OK;
  std::vector<int64_t> csc_off;
  exclusive_scan_host(slot_miss, csc_off);
  CO_CUDA(cudaMalloc(&d_sc, sizeof(int64_t) * h->n_pad));
  k_sample_missing_counts<<<grid_of(h->n_pad, 128), 128, 0, st>>>(h->geno_s, h->n_pad,
                                                                   h->n_panels, d_sc); note_launch();
  std::vector<int64_t> samp_miss(h->n_pad);
  e = cudaMemcpyAsync(samp_miss.data(), d_sc, sizeof(int64_t) * h->n_pad, cudaMemcpyDeviceToHost,
                      st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_sc);
  if (e != cudaSuccess) return cuda_status(e, "sample missing counts");
  std::vector<int64_t> csr_off;
  exclusive_scan_host(samp_miss, csr_off);
  CO_CUDA(cudaMalloc(&h->d_csc_off, sizeof(int64_t) * (h->m_pad + 1)));
  CO_CUDA(cudaMalloc(&h->d_csc_idx, sizeof(int32_t) * total));
  CO_CUDA(cudaMalloc(&h->d_csr_off, sizeof(int64_t) * (h->n_pad + 1)));
  CO_CUDA(cudaMalloc(&h->d_csr_idx, sizeof(int32_t) * total));
  h->device_bytes += sizeof(int64_t) * (h->m_pad + h->n_pad + 2) + 2 * sizeof(int32_t) * total;
  CO_CUDA(cudaMemcpyAsync(h->d_csc_off, csc_off.data(), sizeof(int64_t) * (h->m_pad + 1),
                          cudaMemcpyHostToDevice, st));
  CO_CUDA(cudaMemcpyAsync(h->d_csr_off, csr_off.data(), sizeof(int64_t) * (h->n_pad + 1),
                          cudaMemcpyHostToDevice, st));
  k_fill_csc<<<grid_of(h->m_pad, 128), 128, 0, st>>>(h->geno_t, h->m_pad, h->n_chunks,
                                                     h->d_csc_off, h->d_csc_idx); note_launch();
  k_fill_csr<<<grid_of(h->n_pad, 128), 128, 0, st>>>(h->geno_s, h->n_pad, h->n_panels,
                                                     h->d_csr_off, h->d_csr_idx); note_launch();
  CO_CUDA(cudaGetLastError());
  CO_CUDA(cudaStreamSynchronize(st));
  return COHERIT_OK;
}

// Statistics of one slot.  With override_mean/inv (host, cache order) the
// given standardisation is installed and the trace atoms use the
// standardised sums of squares of the observed genotypes
// (geno_stream.py:1482-1503); otherwise the FP32 reference formulas are
// evaluated on the device and the atoms use the observed counts.
int compute_slot_stats(coherit_geno* h, StatsSlot& s, const float* override_mean,
                       const float* override_inv, float* mean_out, float* inv_out,
                       int32_t* count_out, cudaStream_t st) {
  const int64_t mp = h->m_pad;
  int64_t* d_cnt = nullptr;
  CO_CUDA(cudaMalloc(&d_cnt, sizeof(int64_t) * mp * 3));
  int64_t* d_n1 = d_cnt;
  int64_t* d_n2 = d_cnt + mp;
  int64_t* d_n3 = d_cnt + 2 * mp;
  k_slot_counts<<<grid_of(mp, 128), 128, 0, st>>>(h->geno_t, mp, h->n_chunks, s.tmask, d_n1, d_n2,
                                                  d_n3); note_launch();
  std::vector<int32_t> snp_of_slot(mp);
  std::vector<float> mean(mp, 0.f), inv(mp, 0.f);
  std::vector<int64_t> n1(mp), n2(mp), n3(mp);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && override_mean == nullptr) {
    k_slot_stats<<<grid_of(mp, 256), 256, 0, st>>>(mp, s.n_sub, d_n1, d_n2, d_n3,
                                                   h->d_snp_of_slot, s.mean, s.inv); note_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(mean.data(), s.mean, sizeof(float) * mp, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(inv.data(), s.inv, sizeof(float) * mp, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(snp_of_slot.data(), h->d_snp_of_slot, sizeof(int32_t) * mp,
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(n1.data(), d_n1, sizeof(int64_t) * mp, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(n2.data(), d_n2, sizeof(int64_t) * mp, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(n3.data(), d_n3, sizeof(int64_t) * mp, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_cnt);
  if (e != cudaSuccess) return cuda_status(e, "slot statistics");
  if (override_mean != nullptr) {
    for (int64_t j = 0; j < mp; ++j) {
      const int32_t snp = snp_of_slot[j];
      mean[j] = snp < 0 ? 0.f : override_mean[snp];
      inv[j] = snp < 0 ? 0.f : override_inv[snp];
    }
    CO_CUDA(cudaMemcpyAsync(s.mean, mean.data(), sizeof(float) * mp, cudaMemcpyHostToDevice, st));
    CO_CUDA(cudaMemcpyAsync(s.inv, inv.data(), sizeof(float) * mp, cudaMemcpyHostToDevice, st));
    CO_CUDA(cudaStreamSynchronize(st));
  }
  {
    // Segment sums of diff over the slot's samples, exact in FP64 from the
    // integer counts and the installed FP32 mean.  The operator's first
    // contraction shifts V by its mean over each segment and adds
    // sum_z shift_z * dsum_z back, so no large FP32 running sums occur for
    // columns with an offset or a trend.
    const int ns = static_cast<int>(n_segments(h->n_chunks));
    k_slot_seg_dsum<<<grid_of(mp, 128), 128, 0, st>>>(h->geno_t, mp, h->n_chunks, s.tmask, s.mean,
                                                      s.nseg, h->d_snp_of_slot, ns, s.dseg,
                                                      s.dsum);
    note_launch();
    CO_CUDA(cudaGetLastError());
    CO_CUDA(cudaStreamSynchronize(st));
  }
  // Summaries: m_eff and mean-diagonal atoms per component (FP64 host sums).
  s.comp_eff.assign(h->G, 0.0);
  s.comp_atom.assign(h->G, 0.0);
  std::vector<double> comp_mass(h->G, 0.0);
  double mass_total = 0.0;
  s.eff_total = 0.0;
  for (int g = 0; g < h->G; ++g) {
    for (int64_t j = h->comp_slot_start[g]; j < h->comp_slot_start[g] + h->comp_m[g]; ++j) {
      if (!(inv[j] > 0.f)) continue;
      const double cnt = static_cast<double>(s.n_sub - n3[j]);
      double mass;
      if (override_mean != nullptr) {
        const double s1 = static_cast<double>(n1[j] + 2 * n2[j]);
        const double s2 = static_cast<double>(n1[j] + 4 * n2[j]);
        const double mu = mean[j], iv = inv[j];
        mass = std::max(s2 - 2.0 * mu * s1 + cnt * mu * mu, 0.0) * iv * iv;
      } else {
        mass = cnt;
      }
      s.comp_eff[g] += 1.0;
      comp_mass[g] += mass;
    }
    s.eff_total += s.comp_eff[g];
    mass_total += comp_mass[g];
    s.comp_atom[g] = s.comp_eff[g] > 0.0
                         ? comp_mass[g] / (static_cast<double>(s.n_sub) * s.comp_eff[g])
                         : 0.0;
  }
  s.atom_total = s.eff_total > 0.0 ? mass_total / (static_cast<double>(s.n_sub) * s.eff_total) : 0.0;
  for (int64_t j = 0; j < mp; ++j) {
    const int32_t snp = snp_of_slot[j];
    if (snp < 0) continue;
    if (mean_out) mean_out[snp] = mean[j];
    if (inv_out) inv_out[snp] = inv[j];
    if (count_out) count_out[snp] = static_cast<int32_t>(s.n_sub - n3[j]);
  }
  return COHERIT_OK;
}

int exact_diag_launch(coherit_geno* h, const StatsSlot& s, float* out, cudaStream_t st) {
  const double inv_eff = s.eff_total > 0.0 ? 1.0 / s.eff_total : 0.0;
  if (h->n > 0)
    k_exact_diag<<<grid_of(h->n, 128), 128, 0, st>>>(h->geno_s, h->n, h->n_panels, s.mean, s.inv,
                                                     s.row_mask, inv_eff, out); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

// ------------------------------------------------------------ handle helpers

static int alloc_common(coherit_geno* h, int64_t n, const std::vector<int64_t>& comp_m,
                        int device) {
  h->device = device;
  h->n = n;
  h->G = static_cast<int32_t>(comp_m.size());
  h->comp_m = comp_m;
  h->comp_slot_start.assign(h->G + 1, 0);
  h->comp_snp_start.assign(h->G + 1, 0);
  for (int g = 0; g < h->G; ++g) {
    h->comp_slot_start[g + 1] = h->comp_slot_start[g] + round_up(comp_m[g], kAlign);
    h->comp_snp_start[g + 1] = h->comp_snp_start[g] + comp_m[g];
  }
  h->m = h->comp_snp_start[h->G];
  h->m_pad = round_up(std::max<int64_t>(h->comp_slot_start[h->G], 1), kAlign);
  h->n_pad = round_up(std::max<int64_t>(n, 1), kAlign);
  h->n_panels = h->m_pad / kPanel;
  h->n_chunks = h->n_pad / kPanel;
  h->n_stiles = h->n_pad / kTile;
  h->n_ttiles = h->m_pad / kTile;
  const size_t gbytes = static_cast<size_t>(h->n_pad) * static_cast<size_t>(h->m_pad) / 4;
  CO_CUDA(cudaSetDevice(device));
  int sm = 0;
  CO_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device));
  h->sm_count = sm;
  int v = 0;
  CO_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  h->smem_optin = v;
  CO_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device));
  h->smem_per_sm = v;
  CO_CUDA(cudaMalloc(&h->geno_s, gbytes));
  CO_CUDA(cudaMalloc(&h->geno_t, gbytes));
  CO_CUDA(cudaMalloc(&h->d_comp_of_slot, sizeof(int32_t) * h->m_pad));
  CO_CUDA(cudaMalloc(&h->d_snp_of_slot, sizeof(int32_t) * h->m_pad));
  CO_CUDA(cudaMalloc(&h->d_slot_of_snp, sizeof(int64_t) * std::max<int64_t>(h->m, 1)));
  CO_CUDA(cudaMalloc(&h->d_err, sizeof(int)));
  CO_CUDA(cudaMalloc(&h->d_comp_slot_start, sizeof(int64_t) * (h->G + 1)));
  CO_CUDA(cudaMemcpy(h->d_comp_slot_start, h->comp_slot_start.data(), sizeof(int64_t) * (h->G + 1),
                     cudaMemcpyHostToDevice));
  CO_CUDA(cudaMemset(h->d_err, 0, sizeof(int)));
  h->device_bytes = static_cast<int64_t>(2 * gbytes) + 16 * h->m_pad;
  std::vector<int32_t> comp_of_slot(h->m_pad, h->G - 1), snp_of_slot(h->m_pad, -1);
  std::vector<int64_t> slot_of_snp(std::max<int64_t>(h->m, 1), 0);
  for (int g = 0; g < h->G; ++g) {
    for (int64_t j = h->comp_slot_start[g]; j < h->comp_slot_start[g + 1]; ++j) comp_of_slot[j] = g;
    for (int64_t t = 0; t < comp_m[g]; ++t) {
      const int64_t slot = h->comp_slot_start[g] + t;
      const int64_t snp = h->comp_snp_start[g] + t;
      snp_of_slot[slot] = static_cast<int32_t>(snp);
      slot_of_snp[snp] = slot;
    }
  }
  CO_CUDA(cudaMemcpy(h->d_comp_of_slot, comp_of_slot.data(), sizeof(int32_t) * h->m_pad,
                     cudaMemcpyHostToDevice));
  CO_CUDA(cudaMemcpy(h->d_snp_of_slot, snp_of_slot.data(), sizeof(int32_t) * h->m_pad,
                     cudaMemcpyHostToDevice));
  CO_CUDA(cudaMemcpy(h->d_slot_of_snp, slot_of_snp.data(),
                     sizeof(int64_t) * std::max<int64_t>(h->m, 1), cudaMemcpyHostToDevice));
  return COHERIT_OK;
}

static int init_slot(coherit_geno* h, int32_t slot, const uint8_t* sample_mask, cudaStream_t st) {
  if (slot >= static_cast<int32_t>(h->slots.size())) h->slots.resize(slot + 1);
  StatsSlot& s = h->slots[slot];
  if (!s.used) {
    CO_CUDA(cudaMalloc(&s.mean, sizeof(float) * h->m_pad));
    CO_CUDA(cudaMalloc(&s.inv, sizeof(float) * h->m_pad));
    const int64_t ns = n_segments(h->n_chunks);
    CO_CUDA(cudaMalloc(&s.dsum, sizeof(float) * h->m_pad));
    CO_CUDA(cudaMalloc(&s.dseg, sizeof(float) * h->m_pad * ns));
    CO_CUDA(cudaMalloc(&s.nseg, sizeof(float) * ns));
    s.used = true;
  }
  if (s.row_mask) { cudaFree(s.row_mask); s.row_mask = nullptr; }
  if (s.tmask) { cudaFree(s.tmask); s.tmask = nullptr; }
  s.n_sub = h->n;
  const int64_t seg_len = static_cast<int64_t>(kSegChunks) * kPanel;
  std::vector<float> nseg(n_segments(h->n_chunks), 0.f);
  if (sample_mask == nullptr)
    for (int64_t i = 0; i < h->n; ++i) nseg[i / seg_len] += 1.f;
  if (sample_mask != nullptr) {
    std::vector<uint8_t> rm(h->n_pad, 0);
    int64_t cnt = 0;
    for (int64_t i = 0; i < h->n; ++i) {
      rm[i] = sample_mask[i] ? 1 : 0;
      cnt += rm[i];
      nseg[i / seg_len] += rm[i];
    }
    CO_CHECK(cnt > 0, COHERIT_E_SHAPE, "sample_mask selects no samples");
    s.n_sub = cnt;
    CO_CUDA(cudaMalloc(&s.row_mask, h->n_pad));
    CO_CUDA(cudaMalloc(&s.tmask, sizeof(uint32_t) * 4 * h->n_chunks));
    CO_CUDA(cudaMemcpyAsync(s.row_mask, rm.data(), h->n_pad, cudaMemcpyHostToDevice, st));
    k_build_tmask<<<grid_of(h->n_chunks, 128), 128, 0, st>>>(s.row_mask, h->n, h->n_chunks,
                                                             s.tmask); note_launch();
    CO_CUDA(cudaGetLastError());
  }
  // Segment sample counts (exact integers in FP32: a segment holds 4,096).
  CO_CUDA(cudaMemcpyAsync(s.nseg, nseg.data(), sizeof(float) * nseg.size(),
                          cudaMemcpyHostToDevice, st));
  CO_CUDA(cudaStreamSynchronize(st));
  return COHERIT_OK;
}

static void free_slot(StatsSlot& s) {
  if (s.mean) cudaFree(s.mean);
  if (s.inv) cudaFree(s.inv);
  if (s.dsum) cudaFree(s.dsum);
  if (s.dseg) cudaFree(s.dseg);
  if (s.nseg) cudaFree(s.nseg);
  if (s.row_mask) cudaFree(s.row_mask);
  if (s.tmask) cudaFree(s.tmask);
  s = StatsSlot();
}

static void free_handle(coherit_geno* h) {
  if (h == nullptr) return;
  cudaSetDevice(h->device);
  cudaDeviceSynchronize();
  for (auto& s : h->slots) free_slot(s);
  void* ptrs[] = {h->geno_s,    h->geno_t,    h->d_comp_of_slot, h->d_snp_of_slot,
                  h->d_slot_of_snp, h->d_csc_off, h->d_csc_idx,   h->d_csr_off,
                  h->d_csr_idx, h->ws.base,   h->d_err,         h->d_comp_slot_start};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete h;
}

static int finish_create(coherit_geno* h, cudaStream_t st) {
  int rc = build_missing_lists(h, st);
  if (rc != COHERIT_OK) return rc;
  rc = init_slot(h, 0, nullptr, st);
  if (rc != COHERIT_OK) return rc;
  return compute_slot_stats(h, h->slots[0], nullptr, nullptr, nullptr, nullptr, nullptr, st);
}

}  // namespace coherit

using namespace coherit;

extern "C" {

const char* coherit_last_error(void) { return g_last_error.c_str(); }

int coherit_version(void) { return 1; }

int64_t coherit_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int coherit_device_info(int dev, int* sm_major, int* sm_minor, int* n_sm, int64_t* hbm_bytes) {
  cudaDeviceProp prop;
  CO_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (sm_major) *sm_major = prop.major;
  if (sm_minor) *sm_minor = prop.minor;
  if (n_sm) *n_sm = prop.multiProcessorCount;
  if (hbm_bytes) *hbm_bytes = static_cast<int64_t>(prop.totalGlobalMem);
  return COHERIT_OK;
}

int coherit_geno_create_packed(const uint8_t* packed, int64_t n, int32_t n_calls,
                               const int32_t* call_widths, const int32_t* call_component_ids,
                               int32_t n_components, int packed_on_device, int device,
                               void* stream, coherit_geno_t** out) {
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "out handle pointer is NULL");
  *out = nullptr;
  CO_CHECK(n > 0, COHERIT_E_SHAPE, "genotype matrix must contain at least one sample");
  CO_CHECK(n < (int64_t(1) << 31), COHERIT_E_SHAPE, "n=%lld exceeds 2^31-1", (long long)n);
  CO_CHECK(n_calls > 0, COHERIT_E_SHAPE, "genotype matrix must contain at least one call block");
  CO_CHECK(n_components >= 1, COHERIT_E_SHAPE, "n_components must be >= 1");
  std::vector<int64_t> comp_m(n_components, 0);
  int prev = 0;
  for (int32_t c = 0; c < n_calls; ++c) {
    CO_CHECK(call_widths[c] > 0, COHERIT_E_SHAPE, "call %d has non-positive width", c);
    const int g = call_component_ids ? call_component_ids[c] : 0;
    CO_CHECK(g >= 0 && g < n_components, COHERIT_E_INDEX, "call %d component id %d out of range",
             c, g);
    CO_CHECK(g >= prev, COHERIT_E_SHAPE, "calls of one component must be contiguous");
    prev = g;
    comp_m[g] += call_widths[c];
  }
  coherit_geno* h = new coherit_geno();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = alloc_common(h, n, comp_m, device);
  if (rc != COHERIT_OK) { free_handle(h); return rc; }
  // Per-call offsets and per-SNP (call, column) for the transcode gather.
  std::vector<int64_t> call_off(n_calls);
  std::vector<int32_t> call_pw(n_calls);
  std::vector<int32_t> snp_call(h->m), snp_col(h->m);
  int64_t off = 0, snp = 0;
  for (int32_t c = 0; c < n_calls; ++c) {
    call_off[c] = off;
    call_pw[c] = (call_widths[c] + 3) / 4;
    off += n * call_pw[c];
    for (int32_t t = 0; t < call_widths[c]; ++t, ++snp) {
      snp_call[snp] = c;
      snp_col[snp] = t;
    }
  }
  const int64_t total_bytes = off;
  uint8_t* d_packed = nullptr;
  int64_t* d_call_off = nullptr;
  int32_t *d_call_pw = nullptr, *d_snp_call = nullptr, *d_snp_col = nullptr;
  cudaError_t e = cudaSuccess;
  if (!packed_on_device) {
    e = cudaMalloc(&d_packed, total_bytes);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_packed, packed, total_bytes, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaMalloc(&d_call_off, sizeof(int64_t) * n_calls);
  if (e == cudaSuccess) e = cudaMalloc(&d_call_pw, sizeof(int32_t) * n_calls);
  if (e == cudaSuccess) e = cudaMalloc(&d_snp_call, sizeof(int32_t) * h->m);
  if (e == cudaSuccess) e = cudaMalloc(&d_snp_col, sizeof(int32_t) * h->m);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_call_off, call_off.data(), sizeof(int64_t) * n_calls,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_call_pw, call_pw.data(), sizeof(int32_t) * n_calls,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_snp_call, snp_call.data(), sizeof(int32_t) * h->m,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_snp_col, snp_col.data(), sizeof(int32_t) * h->m, cudaMemcpyHostToDevice,
                        st);
  if (e == cudaSuccess) {
    rc = build_layout_from_ref(h, packed_on_device ? packed : d_packed, d_call_off, d_call_pw,
                               d_snp_call, d_snp_col, st);
    e = cudaStreamSynchronize(st);
  } else {
    rc = cuda_status(e, "upload of packed genotypes");
  }
  if (d_packed) cudaFree(d_packed);
  cudaFree(d_call_off);
  cudaFree(d_call_pw);
  cudaFree(d_snp_call);
  cudaFree(d_snp_col);
  if (rc == COHERIT_OK && e != cudaSuccess) rc = cuda_status(e, "transcode");
  if (rc == COHERIT_OK) rc = finish_create(h, st);
  if (rc != COHERIT_OK) { free_handle(h); return rc; }
  *out = h;
  return COHERIT_OK;
}

int coherit_geno_create_synthetic(int64_t n, int64_t m, const int32_t* component_sizes,
                                  int32_t n_components, uint64_t seed, uint32_t missing_q24,
                                  int device, void* stream, coherit_geno_t** out) {
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "out handle pointer is NULL");
  *out = nullptr;
  CO_CHECK(n > 0 && m > 0, COHERIT_E_SHAPE, "synthetic matrix needs n > 0 and m > 0");
  CO_CHECK(n < (int64_t(1) << 31) && m < (int64_t(1) << 31), COHERIT_E_SHAPE,
           "n and m must be below 2^31");
  std::vector<int64_t> comp_m;
  if (component_sizes == nullptr || n_components <= 1) {
    comp_m.push_back(m);
  } else {
    int64_t tot = 0;
    for (int g = 0; g < n_components; ++g) {
      CO_CHECK(component_sizes[g] > 0, COHERIT_E_SHAPE, "component %d has no SNPs", g);
      comp_m.push_back(component_sizes[g]);
      tot += component_sizes[g];
    }
    CO_CHECK(tot == m, COHERIT_E_SHAPE, "component sizes sum to %lld, expected m=%lld",
             (long long)tot, (long long)m);
  }
  coherit_geno* h = new coherit_geno();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = alloc_common(h, n, comp_m, device);
  if (rc == COHERIT_OK) rc = build_layout_synthetic(h, seed, missing_q24, st);
  if (rc == COHERIT_OK) {
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_status(e, "synthetic genotypes");
  }
  if (rc == COHERIT_OK) rc = finish_create(h, st);
  if (rc != COHERIT_OK) { free_handle(h); return rc; }
  *out = h;
  return COHERIT_OK;
}

int coherit_geno_create_bed(const uint8_t* bed, int64_t bed_bytes, int64_t n_full, int64_t m,
                            const int32_t* keep, int64_t n_keep, const int32_t* component_sizes,
                            int32_t n_components, int device, void* stream,
                            coherit_geno_t** out) {
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "out handle pointer is NULL");
  *out = nullptr;
  CO_CHECK(bed != nullptr && n_full > 0 && m > 0, COHERIT_E_SHAPE,
           "BED input needs a buffer, n > 0 and m > 0");
  const int64_t bps = (n_full + 3) / 4;
  CO_CHECK(bed_bytes >= 3 + bps * m, COHERIT_E_SHAPE,
           "BED buffer holds %lld bytes, expected %lld for n=%lld, m=%lld",
           (long long)bed_bytes, (long long)(3 + bps * m), (long long)n_full, (long long)m);
  CO_CHECK(bed[0] == 0x6C && bed[1] == 0x1B && bed[2] == 0x01, COHERIT_E_SHAPE,
           "Not a valid SNP-major BED file");
  const int64_t n = keep ? n_keep : n_full;
  CO_CHECK(n > 0 && n < (int64_t(1) << 31), COHERIT_E_SHAPE, "sample count %lld out of range",
           (long long)n);
  if (keep)
    for (int64_t i = 0; i < n; ++i)
      CO_CHECK(keep[i] >= 0 && keep[i] < n_full, COHERIT_E_INDEX, "kept sample %lld out of range",
               (long long)i);
  std::vector<int64_t> comp_m;
  if (component_sizes == nullptr || n_components <= 1) {
    comp_m.push_back(m);
  } else {
    int64_t tot = 0;
    for (int g = 0; g < n_components; ++g) {
      CO_CHECK(component_sizes[g] > 0, COHERIT_E_SHAPE, "component %d has no SNPs", g);
      comp_m.push_back(component_sizes[g]);
      tot += component_sizes[g];
    }
    CO_CHECK(tot <= m, COHERIT_E_SHAPE, "components cover %lld SNPs, the BED has %lld",
             (long long)tot, (long long)m);
  }
  coherit_geno* h = new coherit_geno();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = alloc_common(h, n, comp_m, device);
  if (rc != COHERIT_OK) { free_handle(h); return rc; }
  // Cache SNP s of component g sits at slot comp_slot_start[g] + (s - comp_snp_start[g]).
  std::vector<int32_t> slot_of_snp(h->m);
  for (int g = 0; g < h->G; ++g)
    for (int64_t s = h->comp_snp_start[g]; s < h->comp_snp_start[g + 1]; ++s)
      slot_of_snp[s] = static_cast<int32_t>(h->comp_slot_start[g] + (s - h->comp_snp_start[g]));
  int32_t* d_keep = nullptr;
  if (keep) {
    cudaError_t e = cudaMalloc(&d_keep, sizeof(int32_t) * n);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_keep, keep, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { cudaFree(d_keep); free_handle(h); return cuda_status(e, "keep list"); }
  }
  rc = build_layout_from_bed(h, bed + 3, bps, d_keep, slot_of_snp, st);
  if (d_keep) {
    cudaStreamSynchronize(st);
    cudaFree(d_keep);
  }
  if (rc == COHERIT_OK) rc = finish_create(h, st);
  if (rc != COHERIT_OK) { free_handle(h); return rc; }
  *out = h;
  return COHERIT_OK;
}

int coherit_ldblock_records(int64_t n_rows, int64_t m, int32_t block, uint64_t seed,
                            const float* thresholds, const float* rho, const float* sfac,
                            const float* quantiles, uint8_t* out, void* stream) {
  CO_CHECK(n_rows > 0 && m > 0 && block > 0, COHERIT_E_SHAPE,
           "LD-block records need n_rows > 0, m > 0 and block > 0");
  CO_CHECK(thresholds && rho && sfac && quantiles && out, COHERIT_E_SHAPE,
           "LD-block records need device tables and an output buffer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t bps = (n_rows + 3) / 4;
  const int64_t work = bps * ((m + block - 1) / block);
  k_ldblock_records<<<grid_of(work, 256), 256, 0, st>>>(out, n_rows, bps, m, block, seed,
                                                        thresholds, rho, sfac, quantiles,
                                                        nullptr); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

int coherit_geno_create_ldblock(int64_t n, int64_t m, int32_t block, uint64_t seed,
                                const float* thresholds, const float* rho, const float* sfac,
                                const float* quantiles, const int64_t* cache_to_source,
                                const int32_t* component_sizes, int32_t n_components, int device,
                                void* stream, coherit_geno_t** out) {
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "out handle pointer is NULL");
  *out = nullptr;
  CO_CHECK(n > 0 && m > 0 && block > 0, COHERIT_E_SHAPE,
           "LD-block genotypes need n > 0, m > 0 and block > 0");
  CO_CHECK(n < (int64_t(1) << 31) && m < (int64_t(1) << 31), COHERIT_E_SHAPE,
           "n and m must be below 2^31");
  CO_CHECK(thresholds && rho && sfac && quantiles, COHERIT_E_SHAPE, "generator tables missing");
  std::vector<int64_t> comp_m;
  if (component_sizes == nullptr || n_components <= 1) {
    comp_m.push_back(m);
  } else {
    int64_t tot = 0;
    for (int g = 0; g < n_components; ++g) {
      CO_CHECK(component_sizes[g] > 0, COHERIT_E_SHAPE, "component %d has no SNPs", g);
      comp_m.push_back(component_sizes[g]);
      tot += component_sizes[g];
    }
    CO_CHECK(tot == m, COHERIT_E_SHAPE, "component sizes sum to %lld, expected m=%lld",
             (long long)tot, (long long)m);
  }
  // Record (= cache position) of every source SNP.
  std::vector<int64_t> rec(m);
  if (cache_to_source) {
    std::vector<uint8_t> seen(m, 0);
    for (int64_t c = 0; c < m; ++c) {
      const int64_t j = cache_to_source[c];
      CO_CHECK(j >= 0 && j < m && !seen[j], COHERIT_E_SHAPE,
               "cache_to_source must be a permutation of 0..m-1");
      seen[j] = 1;
      rec[j] = c;
    }
  } else {
    for (int64_t j = 0; j < m; ++j) rec[j] = j;
  }
  coherit_geno* h = new coherit_geno();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = alloc_common(h, n, comp_m, device);
  if (rc != COHERIT_OK) { free_handle(h); return rc; }
  const int64_t nb = (m + block - 1) / block;
  const int64_t bps = (n + 3) / 4;
  float *d_thr = nullptr, *d_rho = nullptr, *d_s = nullptr, *d_q = nullptr;
  int64_t* d_rec = nullptr;
  uint8_t* d_bed = nullptr;
  cudaError_t e = cudaMalloc(&d_thr, sizeof(float) * m);
  if (e == cudaSuccess) e = cudaMalloc(&d_rho, sizeof(float) * nb);
  if (e == cudaSuccess) e = cudaMalloc(&d_s, sizeof(float) * nb);
  if (e == cudaSuccess) e = cudaMalloc(&d_q, sizeof(float) * 4096);
  if (e == cudaSuccess) e = cudaMalloc(&d_rec, sizeof(int64_t) * m);
  if (e == cudaSuccess) e = cudaMalloc(&d_bed, static_cast<size_t>(m) * bps);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_thr, thresholds, sizeof(float) * m, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_rho, rho, sizeof(float) * nb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_s, sfac, sizeof(float) * nb, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_q, quantiles, sizeof(float) * 4096, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_rec, rec.data(), sizeof(int64_t) * m, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    k_ldblock_records<<<grid_of(bps * nb, 256), 256, 0, st>>>(d_bed, n, bps, m, block, seed, d_thr,
                                                             d_rho, d_s, d_q, d_rec); note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemsetAsync(h->geno_s, 0, static_cast<size_t>(h->n_pad) * h->m_pad / 4, st);
  if (e == cudaSuccess && h->n_panels > 0) {
    k_build_s_from_bed<<<grid_of(n * h->n_panels, 256), 256, 0, st>>>(
        h->geno_s, n, h->n_pad, h->n_panels, d_bed, bps, 0, m, nullptr, h->d_snp_of_slot, 0,
        h->n_panels); note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_thr); cudaFree(d_rho); cudaFree(d_s); cudaFree(d_q); cudaFree(d_rec); cudaFree(d_bed);
  if (e != cudaSuccess) { free_handle(h); return cuda_status(e, "LD-block genotypes"); }
  rc = build_copy_t(h, st);
  if (rc == COHERIT_OK) rc = finish_create(h, st);
  if (rc != COHERIT_OK) { free_handle(h); return rc; }
  *out = h;
  return COHERIT_OK;
}

int coherit_geno_destroy(coherit_geno_t* h) {
  free_handle(h);
  return COHERIT_OK;
}

int coherit_geno_info(const coherit_geno_t* h, int64_t* n, int64_t* m, int64_t* n_pad,
                      int64_t* m_pad, int32_t* n_components, int64_t* n_missing,
                      int64_t* device_bytes) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  if (n) *n = h->n;
  if (m) *m = h->m;
  if (n_pad) *n_pad = h->n_pad;
  if (m_pad) *m_pad = h->m_pad;
  if (n_components) *n_components = h->G;
  if (n_missing) *n_missing = h->n_missing;
  if (device_bytes) *device_bytes = h->device_bytes + static_cast<int64_t>(h->ws.bytes);
  return COHERIT_OK;
}

int coherit_geno_read_packed(coherit_geno_t* h, int64_t snp_start, int32_t width,
                             uint8_t* out_host, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(snp_start >= 0 && width > 0 && snp_start + width <= h->m, COHERIT_E_SHAPE,
           "SNP range [%lld, %lld) outside [0, %lld)", (long long)snp_start,
           (long long)(snp_start + width), (long long)h->m);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t bytes = h->n * ((width + 3) / 4);
  uint8_t* d = nullptr;
  CO_CUDA(cudaMalloc(&d, bytes));
  k_read_packed<<<grid_of(bytes, 256), 256, 0, st>>>(d, h->geno_s, h->n, h->n_panels,
                                                     h->d_slot_of_snp, snp_start, width); note_launch();
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_host, d, bytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e, "read_packed");
  return COHERIT_OK;
}

int coherit_geno_extract_columns(coherit_geno_t* h, int32_t slot, const int64_t* snp_idx,
                                 int32_t count, float* out, int64_t ldo, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(slot >= 0 && slot < static_cast<int32_t>(h->slots.size()) && h->slots[slot].used,
           COHERIT_E_INDEX, "stats slot %d is not initialised", slot);
  CO_CHECK(count >= 0 && ldo >= count, COHERIT_E_SHAPE, "need 0 <= count <= ldo");
  if (count == 0) return COHERIT_OK;
  CO_CHECK(snp_idx != nullptr && out != nullptr, COHERIT_E_SHAPE, "snp_idx and out are required");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned gy = static_cast<unsigned>(std::min<int64_t>((h->n + 7) / 8, 8192));
  k_extract_std<<<dim3(static_cast<unsigned>((count + 31) / 32), gy), dim3(32, 8), 0, st>>>(
      out, ldo, snp_idx, count, h->geno_t, h->n, h->m, h->n_chunks, h->d_slot_of_snp,
      h->slots[slot].mean, h->slots[slot].inv); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

int coherit_geno_compute_stats(coherit_geno_t* h, int32_t slot, const uint8_t* sample_mask,
                               float* mean_out, float* inv_sd_out, int32_t* count_out,
                               void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(slot >= 0 && slot < 1 << 20, COHERIT_E_INDEX, "stats slot %d out of range", slot);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = init_slot(h, slot, sample_mask, st);
  if (rc != COHERIT_OK) return rc;
  return compute_slot_stats(h, h->slots[slot], nullptr, nullptr, mean_out, inv_sd_out, count_out,
                            st);
}

int coherit_geno_set_stats(coherit_geno_t* h, int32_t slot, const uint8_t* sample_mask,
                           const float* mean, const float* inv_sd, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(slot >= 0 && slot < 1 << 20, COHERIT_E_INDEX, "stats slot %d out of range", slot);
  CO_CHECK(mean != nullptr && inv_sd != nullptr, COHERIT_E_SHAPE, "mean and inv_sd are required");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = init_slot(h, slot, sample_mask, st);
  if (rc != COHERIT_OK) return rc;
  return compute_slot_stats(h, h->slots[slot], mean, inv_sd, nullptr, nullptr, nullptr, st);
}

int coherit_geno_release_stats(coherit_geno_t* h, int32_t slot) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(slot > 0 && slot < static_cast<int32_t>(h->slots.size()), COHERIT_E_INDEX,
           "stats slot %d cannot be released", slot);
  cudaStreamSynchronize(nullptr);
  free_slot(h->slots[slot]);
  return COHERIT_OK;
}

int coherit_geno_stats_summary(const coherit_geno_t* h, int32_t slot, double* comp_eff,
                               double* comp_atom, double* eff_total, double* atom_total) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(slot >= 0 && slot < static_cast<int32_t>(h->slots.size()) && h->slots[slot].used,
           COHERIT_E_INDEX, "stats slot %d is not initialised", slot);
  const StatsSlot& s = h->slots[slot];
  for (int g = 0; g < h->G; ++g) {
    if (comp_eff) comp_eff[g] = s.comp_eff[g];
    if (comp_atom) comp_atom[g] = s.comp_atom[g];
  }
  if (eff_total) *eff_total = s.eff_total;
  if (atom_total) *atom_total = s.atom_total;
  return COHERIT_OK;
}

int coherit_geno_exact_diag(coherit_geno_t* h, int32_t slot, float* out, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(slot >= 0 && slot < static_cast<int32_t>(h->slots.size()) && h->slots[slot].used,
           COHERIT_E_INDEX, "stats slot %d is not initialised", slot);
  return exact_diag_launch(h, h->slots[slot], out, static_cast<cudaStream_t>(stream));
}

int coherit_geno_check(coherit_geno_t* h, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int flag = 0;
  CO_CUDA(cudaMemcpyAsync(&flag, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CO_CUDA(cudaStreamSynchronize(st));
  if (flag != 0) {
    CO_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), st));
    CO_CUDA(cudaStreamSynchronize(st));
    set_error("a device wait exceeded its time limit (code %d)", flag);
    return COHERIT_E_TIMEOUT;
  }
  return COHERIT_OK;
}

}  // extern "C"
