// sparse.cu -- rare-variant ("sparse12") genotype operator on per-SNP entry
// lists resident in HBM.
//
// Layout on the device:
//   * col_off[m + 1] (int64): the entries of SNP j are [col_off[j], col_off[j+1]);
//   * entry[nnz] (uint32): (sample << 2) | value, value 1 = het, 2 = hom-alt,
//     3 = missing; samples ascending within a SNP; genotype 0 is not stored
//     (the entry order of sparse_stream.py:570-606);
//   * mean[m], inv[m] (float): the reference FP32 statistics.
//
// Operator.  With x_ij the stored value (1, 2, or mean_j for a missing entry)
// and z_ij = inv_j (x_ij - mean_j), one fused pass per column chunk computes
//   s_j  = inv_j (sum_{p in j} x_p V[row_p] - mean_j sum(V))            (Z^T V)
//   out  = theta_e V + scale (sum_j inv_j x_j s_j^T - 1 c^T),
//   c    = sum_j inv_j mean_j s_j,
// which equals the reference's row_sparse + row_b sum_v + base decomposition
// (kv_impl.py:777-817) term by term.  One warp owns a SNP: it gathers V rows
// of its entries (4L columns per entry, L lanes per entry, 32/L entries in
// flight per step), reduces across the entry lanes, forms s_j in FP64 and
// scatters inv_j x_p s_j back with vector atomics into the L2-resident out.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "coherit_internal.cuh"

struct coherit_sparse {
  int device = 0;
  int64_t n = 0, m = 0, nnz = 0;
  int64_t* d_col_off = nullptr;
  uint32_t* d_entry = nullptr;
  float* d_mean = nullptr;
  float* d_inv = nullptr;
  std::vector<float> mean, inv;
  std::vector<int64_t> n_het, n_hom, n_miss;
  double eff = 0.0, atom = 0.0, diag_base = 0.0;
  double* d_ws = nullptr;  // sum(V)[k_cap] then c[k_cap]
  int32_t k_cap = 0;
  double* d_diag = nullptr;  // n, exact diagonal accumulator
  float* d_stage = nullptr;  // padded copies of V and out for k % 4 != 0 / unaligned rows
  size_t stage_bytes = 0;
  int sm_count = 0;
  int64_t device_bytes = 0;
};

namespace coherit {
namespace {

constexpr int kMaxRows = 1 << 30;  // sample index must fit in 30 bits

inline unsigned blocks_for(int64_t work, int threads, int64_t cap = 0x7FFFFFFF) {
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, cap)));
}

__device__ __forceinline__ uint32_t bed_value(const uint8_t* rec, int64_t src) {
  // BED 00, 01, 10, 11 -> 2 (hom A1), 3 (missing), 1 (het), 0.
  const uint32_t b = (static_cast<uint32_t>(rec[src >> 2]) >> (2 * (src & 3))) & 3u;
  return (0x1Eu >> (2 * b)) & 3u;
}

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Genotype sources of the entry build.  record(w) prepares SNP record w of
// the current chunk, value(r, i) is the stored value (0 = not stored, 1 het,
// 2 hom-alt, 3 missing) of kept sample i.
struct BedRecords {
  const uint8_t* rec0;
  int64_t bps;
  const int32_t* keep;
  __device__ const uint8_t* record(int64_t w) const { return rec0 + w * bps; }
  __device__ uint32_t value(const uint8_t* r, int64_t i) const {
    return bed_value(r, keep ? keep[i] : i);
  }
};

// Counter-based rare-variant generator: MAF ~ U[lo, lo + span) / 2^24 per
// SNP, two Bernoulli(MAF) alleles per sample, optional missing rate.
struct SynthRecords {
  uint64_t seed;
  int64_t s0;
  uint32_t lo, span, miss;
  struct Rec {
    uint64_t key;
    uint32_t maf;
  };
  __device__ Rec record(int64_t w) const {
    return Rec{synth_snp_key(seed, s0 + w), synth_maf_q24_range(seed, s0 + w, lo, span)};
  }
  __device__ uint32_t value(const Rec& r, int64_t i) const {
    return synth_code_keyed(r.key, i, r.maf, miss);
  }
};

// Non-zero genotypes of each SNP record of a chunk: one warp per SNP, each
// lane owning 16 consecutive kept samples per step.
template <class Src>
__global__ void k_rec_count(const Src src, int64_t count, int64_t n, int32_t* __restrict__ nnz) {
  const int64_t w = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= count) return;
  const auto rec = src.record(w);
  int c = 0;
  for (int64_t i0 = 16 * static_cast<int64_t>(lane); i0 < n; i0 += 512) {
    const int64_t hi = min(i0 + 16, n);
    for (int64_t i = i0; i < hi; ++i) c += src.value(rec, i) != 0u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
  if (lane == 0) nnz[w] = c;
}

// Entries of each SNP record in sample order (same ownership as k_rec_count;
// a warp prefix sum of the per-lane counts places each lane's entries).
template <class Src>
__global__ void k_rec_fill(const Src src, int64_t count, int64_t n,
                           const int64_t* __restrict__ col_off, uint32_t* __restrict__ entry) {
  const int64_t w = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= count) return;
  const auto rec = src.record(w);
  int64_t pos = col_off[w];
  for (int64_t base = 0; base < n; base += 512) {
    const int64_t i0 = base + 16 * static_cast<int64_t>(lane);
    const int64_t hi = min(i0 + 16, n);
    uint32_t vals = 0;  // 2 bits per owned sample
    int c = 0;
    for (int64_t i = i0; i < hi; ++i) {
      const uint32_t v = src.value(rec, i);
      vals |= v << (2 * (i - i0));
      c += v != 0u;
    }
    const int incl = warp_incl_scan(c, lane);
    int64_t p = pos + incl - c;
    for (int64_t i = i0; i < hi; ++i) {
      const uint32_t v = (vals >> (2 * (i - i0))) & 3u;
      if (v != 0u) entry[p++] = (static_cast<uint32_t>(i) << 2) | v;
    }
    pos += __shfl_sync(0xFFFFFFFFu, incl, 31);
  }
}

// Per-SNP het / hom / missing counts from the entries and the reference FP32
// statistics (sparse_stream.py:518-567, :726-735).
__global__ void k_col_stats(const int64_t* __restrict__ col_off, const uint32_t* __restrict__ entry,
                            int64_t m, int64_t n, int64_t* __restrict__ cnt3,
                            float* __restrict__ mean, float* __restrict__ inv) {
  const int64_t j = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= m) return;
  long long a[3] = {0, 0, 0};
  for (int64_t p = col_off[j] + lane; p < col_off[j + 1]; p += 32) {
    const uint32_t v = entry[p] & 3u;
    a[0] += v == 1u;
    a[1] += v == 2u;
    a[2] += v == 3u;
  }
#pragma unroll
  for (int t = 0; t < 3; ++t)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a[t] += __shfl_xor_sync(0xFFFFFFFFu, a[t], o);
  if (lane == 0) {
    cnt3[3 * j] = a[0];
    cnt3[3 * j + 1] = a[1];
    cnt3[3 * j + 2] = a[2];
    ref_fp32_standardize(n, a[0], a[1], a[2], mean[j], inv[j]);
  }
}

// Column sums of V in FP64 (atomically combined per block) and, for the
// operator, out = theta_e V.  Block (32, 8): x = column, y = row stride.
__global__ void k_prep(const float* __restrict__ V, int64_t ldv, int64_t n, int32_t k,
                       float theta_e, float* __restrict__ out, int64_t ldo,
                       double* __restrict__ sumv) {
  __shared__ double red[8][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  double acc = 0.0;
  if (c < k) {
    for (int64_t i = blockIdx.y * 8 + threadIdx.y; i < n; i += static_cast<int64_t>(gridDim.y) * 8) {
      const float v = V[i * ldv + c];
      acc += static_cast<double>(v);
      if (out != nullptr) out[i * ldo + c] = theta_e * v;
    }
  }
  red[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && c < k) {
    double t = 0.0;
#pragma unroll
    for (int y = 0; y < 8; ++y) t += red[y][threadIdx.x];
    atomicAdd(sumv + c, t);
  }
}

__device__ __forceinline__ float entry_x(uint32_t e, float mu) {
  const uint32_t v = e & 3u;
  return v == 3u ? mu : static_cast<float>(v);
}

__device__ __forceinline__ void fma4(float4& a, float x, const float4& v) {
  a.x = fmaf(x, v.x, a.x);
  a.y = fmaf(x, v.y, a.y);
  a.z = fmaf(x, v.z, a.z);
  a.w = fmaf(x, v.w, a.w);
}

struct ApplyArgs {
  const int64_t* col_off;
  const uint32_t* entry;
  const float* mean;
  const float* inv;
  int64_t m;
  const float* V;
  int64_t ldv;
  int32_t k;
  const double* sumv;
  double scale;
  float* out;
  int64_t ldo;
  double* corr;
};

__device__ __forceinline__ float4 gather4(const float* p) {
  return __ldg(reinterpret_cast<const float4*>(p));
}

__device__ __forceinline__ void scatter4(float* p, float4 v) {
  atomicAdd(reinterpret_cast<float4*>(p), v);
}

// KV = false: out (m x k) = scale Z^T V.  KV = true: out (n x k) += scale Z Z^T V
// without the rank-one term, whose vector c is accumulated into corr.
// Requires k % 4 == 0 and 16-byte aligned rows of V and out (the host
// stages other blocks through padded buffers), so every access is one
// 128-bit gather / store / atomic add.  Lanes whose 4 columns lie beyond k
// skip the entry loops entirely, so the loops of the active lanes stay
// branch-free with 4 gathers in flight.
template <int L, bool KV>
__global__ void __launch_bounds__(256) k_apply(const ApplyArgs a) {
  constexpr int E = 32 / L;  // entries in flight per warp step
  const int lane = threadIdx.x & 31;
  const int g = lane / L, q = lane % L;
  const int64_t w0 = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int c0 = 0; c0 < a.k; c0 += 4 * L) {
    const int col = c0 + 4 * q;
    const bool active = col < a.k;
    double sv[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) sv[t] = active ? a.sumv[col + t] : 0.0;
    double cacc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t j = w0; j < a.m; j += nw) {
      const float iv = a.inv[j];
      if (!(iv != 0.f)) {
        if (!KV && g == 0 && active)
          *reinterpret_cast<float4*>(a.out + j * a.ldo + col) = make_float4(0.f, 0.f, 0.f, 0.f);
        continue;
      }
      const float mu = a.mean[j];
      const int64_t p0 = a.col_off[j], p1 = a.col_off[j + 1];
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      if (active) {
        const float* Vc = a.V + col;
        int64_t p = p0 + g;
        for (; p + 3 * E < p1; p += 4 * E) {
          const uint32_t e0 = __ldg(a.entry + p), e1 = __ldg(a.entry + p + E);
          const uint32_t e2 = __ldg(a.entry + p + 2 * E), e3 = __ldg(a.entry + p + 3 * E);
          const float4 v0 = gather4(Vc + static_cast<int64_t>(e0 >> 2) * a.ldv);
          const float4 v1 = gather4(Vc + static_cast<int64_t>(e1 >> 2) * a.ldv);
          const float4 v2 = gather4(Vc + static_cast<int64_t>(e2 >> 2) * a.ldv);
          const float4 v3 = gather4(Vc + static_cast<int64_t>(e3 >> 2) * a.ldv);
          fma4(acc, entry_x(e0, mu), v0);
          fma4(acc, entry_x(e1, mu), v1);
          fma4(acc, entry_x(e2, mu), v2);
          fma4(acc, entry_x(e3, mu), v3);
        }
        for (; p < p1; p += E) {
          const uint32_t e = __ldg(a.entry + p);
          fma4(acc, entry_x(e, mu), gather4(Vc + static_cast<int64_t>(e >> 2) * a.ldv));
        }
      }
#pragma unroll
      for (int o = L; o < 32; o <<= 1) {
        acc.x += __shfl_xor_sync(0xFFFFFFFFu, acc.x, o);
        acc.y += __shfl_xor_sync(0xFFFFFFFFu, acc.y, o);
        acc.z += __shfl_xor_sync(0xFFFFFFFFu, acc.z, o);
        acc.w += __shfl_xor_sync(0xFFFFFFFFu, acc.w, o);
      }
      if (!active) continue;
      const double div = static_cast<double>(iv), dmu = static_cast<double>(mu);
      const double s0 = div * (static_cast<double>(acc.x) - dmu * sv[0]);
      const double s1 = div * (static_cast<double>(acc.y) - dmu * sv[1]);
      const double s2 = div * (static_cast<double>(acc.z) - dmu * sv[2]);
      const double s3 = div * (static_cast<double>(acc.w) - dmu * sv[3]);
      if (!KV) {
        if (g == 0)
          *reinterpret_cast<float4*>(a.out + j * a.ldo + col) =
              make_float4(static_cast<float>(a.scale * s0), static_cast<float>(a.scale * s1),
                          static_cast<float>(a.scale * s2), static_cast<float>(a.scale * s3));
        continue;
      }
      const double f = a.scale * div;
      const float4 wv = make_float4(static_cast<float>(f * s0), static_cast<float>(f * s1),
                                    static_cast<float>(f * s2), static_cast<float>(f * s3));
      if (g == 0) {
        cacc[0] += f * dmu * s0;
        cacc[1] += f * dmu * s1;
        cacc[2] += f * dmu * s2;
        cacc[3] += f * dmu * s3;
      }
      float* Oc = a.out + col;
      int64_t p = p0 + g;
      for (; p + 3 * E < p1; p += 4 * E) {
        const uint32_t e0 = __ldg(a.entry + p), e1 = __ldg(a.entry + p + E);
        const uint32_t e2 = __ldg(a.entry + p + 2 * E), e3 = __ldg(a.entry + p + 3 * E);
        float x = entry_x(e0, mu);
        scatter4(Oc + static_cast<int64_t>(e0 >> 2) * a.ldo,
                      make_float4(x * wv.x, x * wv.y, x * wv.z, x * wv.w));
        x = entry_x(e1, mu);
        scatter4(Oc + static_cast<int64_t>(e1 >> 2) * a.ldo,
                      make_float4(x * wv.x, x * wv.y, x * wv.z, x * wv.w));
        x = entry_x(e2, mu);
        scatter4(Oc + static_cast<int64_t>(e2 >> 2) * a.ldo,
                      make_float4(x * wv.x, x * wv.y, x * wv.z, x * wv.w));
        x = entry_x(e3, mu);
        scatter4(Oc + static_cast<int64_t>(e3 >> 2) * a.ldo,
                      make_float4(x * wv.x, x * wv.y, x * wv.z, x * wv.w));
      }
      for (; p < p1; p += E) {
        const uint32_t e = __ldg(a.entry + p);
        const float x = entry_x(e, mu);
        scatter4(Oc + static_cast<int64_t>(e >> 2) * a.ldo,
                      make_float4(x * wv.x, x * wv.y, x * wv.z, x * wv.w));
      }
    }
    if (KV && g == 0 && active) {
#pragma unroll
      for (int t = 0; t < 4; ++t) atomicAdd(a.corr + col + t, cacc[t]);
    }
  }
}

// out[i, c] -= c_c (the rank-one term of the operator).
__global__ void k_finish(float* __restrict__ out, int64_t ldo, int64_t n, int32_t k,
                         const double* __restrict__ corr) {
  const int c = blockIdx.x * 32 + threadIdx.x;
  if (c >= k) return;
  const float cc = static_cast<float>(corr[c]);
  for (int64_t i = blockIdx.y * 8 + threadIdx.y; i < n; i += static_cast<int64_t>(gridDim.y) * 8)
    out[i * ldo + c] -= cc;
}

// Standardised columns: every sample first gets the genotype-0 value
// (0 - mean) inv, then the stored entries overwrite theirs (missing -> 0).
__global__ void k_extract_fill(float* __restrict__ out, int64_t ldo, int64_t n, int32_t count,
                               const int64_t* __restrict__ idx, int64_t m,
                               const float* __restrict__ mean, const float* __restrict__ inv) {
  const int c = blockIdx.x * 32 + threadIdx.x;
  if (c >= count) return;
  const int64_t j = idx[c];
  const bool ok = j >= 0 && j < m;
  const float z0 = ok ? __fmul_rn(__fsub_rn(0.f, mean[j]), inv[j]) : __int_as_float(0x7FC00000);
  for (int64_t i = blockIdx.y * 8 + threadIdx.y; i < n; i += static_cast<int64_t>(gridDim.y) * 8)
    out[i * ldo + c] = z0;
}

__global__ void k_extract_scatter(float* __restrict__ out, int64_t ldo, int32_t count,
                                  const int64_t* __restrict__ idx, int64_t m,
                                  const int64_t* __restrict__ col_off,
                                  const uint32_t* __restrict__ entry,
                                  const float* __restrict__ mean, const float* __restrict__ inv) {
  const int64_t c = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= count) return;
  const int64_t j = idx[c];
  if (j < 0 || j >= m) return;
  const float mu = mean[j], iv = inv[j];
  for (int64_t p = col_off[j] + lane; p < col_off[j + 1]; p += 32) {
    const uint32_t e = entry[p];
    const uint32_t v = e & 3u;
    out[static_cast<int64_t>(e >> 2) * ldo + c] =
        v == 3u ? 0.f : __fmul_rn(__fsub_rn(static_cast<float>(v), mu), iv);
  }
}

// Exact diagonal: per entry z^2 - z0^2 in FP64 added to the sample's total.
__global__ void k_diag_entries(const int64_t* __restrict__ col_off, const uint32_t* __restrict__ entry,
                               int64_t m, const float* __restrict__ mean,
                               const float* __restrict__ inv, double* __restrict__ diag) {
  const int64_t j = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= m) return;
  const float mu = mean[j], iv = inv[j];
  if (!(iv != 0.f)) return;
  const double z0 = static_cast<double>(__fmul_rn(__fsub_rn(0.f, mu), iv));
  for (int64_t p = col_off[j] + lane; p < col_off[j + 1]; p += 32) {
    const uint32_t e = entry[p];
    const uint32_t v = e & 3u;
    const double z = v == 3u ? 0.0 : static_cast<double>(__fmul_rn(__fsub_rn(static_cast<float>(v), mu), iv));
    atomicAdd(diag + (e >> 2), z * z - z0 * z0);
  }
}

__global__ void k_diag_finish(const double* __restrict__ diag, int64_t n, double base, double eff,
                              float* __restrict__ out) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  out[i] = eff > 0.0 ? static_cast<float>((base + diag[i]) / eff) : 0.f;
}

void free_sparse(coherit_sparse* h) {
  if (h == nullptr) return;
  cudaFree(h->d_col_off);
  cudaFree(h->d_entry);
  cudaFree(h->d_mean);
  cudaFree(h->d_inv);
  cudaFree(h->d_ws);
  cudaFree(h->d_diag);
  cudaFree(h->d_stage);
  delete h;
}

int alloc_sparse(coherit_sparse* h, int64_t n, int64_t m, int device) {
  CO_CHECK(n > 0 && n < kMaxRows, COHERIT_E_SHAPE, "sample count %lld out of range (1..2^30-1)",
           (long long)n);
  CO_CHECK(m >= 0, COHERIT_E_SHAPE, "negative SNP count");
  h->device = device;
  h->n = n;
  h->m = m;
  CO_CUDA(cudaSetDevice(device));
  CO_CUDA(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device));
  CO_CUDA(cudaMalloc(&h->d_col_off, sizeof(int64_t) * (m + 1)));
  CO_CUDA(cudaMalloc(&h->d_mean, sizeof(float) * std::max<int64_t>(m, 1)));
  CO_CUDA(cudaMalloc(&h->d_inv, sizeof(float) * std::max<int64_t>(m, 1)));
  h->device_bytes = sizeof(int64_t) * (m + 1) + 2 * sizeof(float) * std::max<int64_t>(m, 1);
  return COHERIT_OK;
}

// Statistics and summaries once the entries are resident: het / hom /
// missing counts, FP32 mean and inverse sd, m_eff = number of SNPs with
// inv > 0 and the mean-diagonal atom sum_valid cnt / (n m_eff)
// (geno_stream.py:1409-1420 with the observed counts as trace mass).
int finish_sparse(coherit_sparse* h, cudaStream_t st) {
  const int64_t m = h->m;
  h->mean.assign(m, 0.f);
  h->inv.assign(m, 0.f);
  h->n_het.assign(m, 0);
  h->n_hom.assign(m, 0);
  h->n_miss.assign(m, 0);
  if (m > 0) {
    int64_t* d_cnt = nullptr;
    CO_CUDA(cudaMalloc(&d_cnt, sizeof(int64_t) * 3 * m));
    k_col_stats<<<blocks_for(m * 32, 256), 256, 0, st>>>(
        h->d_col_off, h->d_entry, m, h->n, d_cnt, h->d_mean, h->d_inv); note_launch();
    std::vector<int64_t> cnt(3 * m);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int64_t) * 3 * m, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->mean.data(), h->d_mean, sizeof(float) * m, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->inv.data(), h->d_inv, sizeof(float) * m, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_cnt);
    if (e != cudaSuccess) return cuda_status(e, "sparse statistics");
    for (int64_t j = 0; j < m; ++j) {
      h->n_het[j] = cnt[3 * j];
      h->n_hom[j] = cnt[3 * j + 1];
      h->n_miss[j] = cnt[3 * j + 2];
    }
  }
  double eff = 0.0, mass = 0.0, base = 0.0;
  for (int64_t j = 0; j < m; ++j) {
    if (!(h->inv[j] > 0.f)) continue;
    eff += 1.0;
    mass += static_cast<double>(h->n - h->n_miss[j]);
    const float z0 = (0.f - h->mean[j]) * h->inv[j];
    base += static_cast<double>(z0) * static_cast<double>(z0);
  }
  h->eff = eff;
  h->atom = eff > 0.0 ? mass / (static_cast<double>(h->n) * eff) : 0.0;
  h->diag_base = base;
  return COHERIT_OK;
}

int ensure_ws(coherit_sparse* h, int32_t k) {
  if (k <= h->k_cap) return COHERIT_OK;
  if (h->d_ws != nullptr) CO_CUDA(cudaDeviceSynchronize());
  cudaFree(h->d_ws);
  h->d_ws = nullptr;
  h->k_cap = 0;
  const int32_t cap = std::max<int32_t>(64, (k + 63) / 64 * 64);
  CO_CUDA(cudaMalloc(&h->d_ws, sizeof(double) * 2 * cap));
  h->k_cap = cap;
  return COHERIT_OK;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// One full wave of a persistent grid: every SM holds as many 256-thread
// blocks of this kernel as its registers allow, and each warp strides over
// the SNPs (a partial second wave of equal-work blocks would idle SMs).
template <int L, bool KV>
void launch_one(int sm_count, int64_t m, const ApplyArgs& a, cudaStream_t st) {
  static const int per_sm = [] {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_apply<L, KV>, 256, 0) !=
            cudaSuccess || nb < 1)
      nb = 1;
    return nb;
  }();
  const unsigned grid = blocks_for(std::max<int64_t>(m, 1) * 32, 256,
                                   static_cast<int64_t>(sm_count) * per_sm);
  k_apply<L, KV><<<grid, 256, 0, st>>>(a);
}

template <bool KV>
int launch_apply(coherit_sparse* h, const ApplyArgs& a, cudaStream_t st) {
  const int k = a.k;
  if (k <= 4)
    launch_one<1, KV>(h->sm_count, h->m, a, st);
  else if (k <= 8)
    launch_one<2, KV>(h->sm_count, h->m, a, st);
  else if (k <= 16)
    launch_one<4, KV>(h->sm_count, h->m, a, st);
  else if (k <= 32)
    launch_one<8, KV>(h->sm_count, h->m, a, st);
  else
    launch_one<16, KV>(h->sm_count, h->m, a, st);
  note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

int ensure_stage(coherit_sparse* h, size_t bytes) {
  if (bytes <= h->stage_bytes) return COHERIT_OK;
  // The old buffer may still be read by queued work.
  if (h->d_stage != nullptr) CO_CUDA(cudaDeviceSynchronize());
  cudaFree(h->d_stage);
  h->d_stage = nullptr;
  h->stage_bytes = 0;
  CO_CUDA(cudaMalloc(&h->d_stage, bytes));
  h->stage_bytes = bytes;
  return COHERIT_OK;
}

int sparse_apply(coherit_sparse* h, bool kv, const float* V, int64_t ldv, int32_t k, double scale,
                 float theta_e, float* out, int64_t ldo, cudaStream_t st) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "sparse handle is NULL");
  CO_CHECK(k >= 0 && ldv >= k && ldo >= k, COHERIT_E_SHAPE, "bad k=%d / ldv=%lld / ldo=%lld", k,
           (long long)ldv, (long long)ldo);
  if (k == 0) return COHERIT_OK;
  CO_CHECK(V != nullptr && out != nullptr, COHERIT_E_SHAPE, "V and out must be device pointers");
  CO_CHECK(static_cast<const void*>(V) != static_cast<const void*>(out), COHERIT_E_SHAPE,
           "out must not alias V");
  CO_CUDA(cudaSetDevice(h->device));
  const int64_t out_rows = kv ? h->n : h->m;
  // The kernels take k % 4 == 0 and 16-byte rows; other blocks go through a
  // zero-padded staging copy of V and of the output.
  const bool direct = k % 4 == 0 && aligned16(V) && ldv % 4 == 0 && aligned16(out) &&
                      ldo % 4 == 0;
  const float* Vr = V;
  float* outr = out;
  int64_t ldvr = ldv, ldor = ldo;
  int32_t kr = k;
  int rc = COHERIT_OK;
  if (!direct) {
    kr = (k + 3) / 4 * 4;
    const size_t vfl = static_cast<size_t>(h->n) * kr;
    rc = ensure_stage(h, sizeof(float) * (vfl + static_cast<size_t>(out_rows) * kr));
    if (rc != COHERIT_OK) return rc;
    float* vs = h->d_stage;
    if (kr != k) CO_CUDA(cudaMemsetAsync(vs, 0, sizeof(float) * vfl, st));
    CO_CUDA(cudaMemcpy2DAsync(vs, sizeof(float) * kr, V, sizeof(float) * ldv, sizeof(float) * k,
                              h->n, cudaMemcpyDeviceToDevice, st));
    Vr = vs;
    outr = h->d_stage + vfl;
    ldvr = ldor = kr;
  }
  rc = ensure_ws(h, kr);
  if (rc != COHERIT_OK) return rc;
  double* sumv = h->d_ws;
  double* corr = h->d_ws + h->k_cap;
  CO_CUDA(cudaMemsetAsync(h->d_ws, 0, sizeof(double) * 2 * h->k_cap, st));
  const dim3 blk(32, 8);
  const dim3 grd(static_cast<unsigned>((kr + 31) / 32),
                 static_cast<unsigned>(std::min<int64_t>((h->n + 63) / 64, 4096)));
  k_prep<<<grd, blk, 0, st>>>(Vr, ldvr, h->n, kr, theta_e, kv ? outr : nullptr, ldor, sumv); note_launch();
  CO_CUDA(cudaGetLastError());
  if (h->m > 0 && h->eff > 0.0) {
    ApplyArgs a{h->d_col_off, h->d_entry, h->d_mean, h->d_inv, h->m, Vr, ldvr, kr, sumv, scale,
                outr, ldor, corr};
    rc = kv ? launch_apply<true>(h, a, st) : launch_apply<false>(h, a, st);
    if (rc != COHERIT_OK) return rc;
    if (kv) {
      k_finish<<<grd, blk, 0, st>>>(outr, ldor, h->n, kr, corr); note_launch();
      CO_CUDA(cudaGetLastError());
    }
  } else if (!kv && h->m > 0) {
    CO_CUDA(cudaMemset2DAsync(outr, sizeof(float) * ldor, 0, sizeof(float) * kr, h->m, st));
  }
  if (!direct && out_rows > 0)
    CO_CUDA(cudaMemcpy2DAsync(out, sizeof(float) * ldo, outr, sizeof(float) * kr,
                              sizeof(float) * k, out_rows, cudaMemcpyDeviceToDevice, st));
  return COHERIT_OK;
}

int upload_entries_from_host(coherit_sparse* h, const int64_t* col_off, const int32_t* rows,
                             const int8_t* vals, cudaStream_t st) {
  const int64_t nnz = col_off[h->m];
  std::vector<uint32_t> packed(static_cast<size_t>(nnz));
  for (int64_t p = 0; p < nnz; ++p)
    packed[p] = (static_cast<uint32_t>(rows[p]) << 2) | static_cast<uint32_t>(vals[p]);
  h->nnz = nnz;
  CO_CUDA(cudaMalloc(&h->d_entry, sizeof(uint32_t) * std::max<int64_t>(nnz, 1)));
  h->device_bytes += sizeof(uint32_t) * std::max<int64_t>(nnz, 1);
  CO_CUDA(cudaMemcpyAsync(h->d_col_off, col_off, sizeof(int64_t) * (h->m + 1),
                          cudaMemcpyHostToDevice, st));
  if (nnz > 0)
    CO_CUDA(cudaMemcpyAsync(h->d_entry, packed.data(), sizeof(uint32_t) * nnz,
                            cudaMemcpyHostToDevice, st));
  CO_CUDA(cudaStreamSynchronize(st));
  return COHERIT_OK;
}

}  // namespace
}  // namespace coherit

using namespace coherit;

extern "C" {

int coherit_sparse_create_bed(const uint8_t* bed, int64_t bed_bytes, int64_t n_full, int64_t m,
                              const int32_t* keep, int64_t n_keep, int device, void* stream,
                              coherit_sparse_t** out) {
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "out handle pointer is NULL");
  *out = nullptr;
  CO_CHECK(bed != nullptr && n_full > 0 && m >= 0, COHERIT_E_SHAPE,
           "BED input needs a buffer, n > 0 and m >= 0");
  const int64_t bps = (n_full + 3) / 4;
  CO_CHECK(bed_bytes >= 3 + bps * m, COHERIT_E_SHAPE,
           "BED buffer holds %lld bytes, expected %lld for n=%lld, m=%lld",
           (long long)bed_bytes, (long long)(3 + bps * m), (long long)n_full, (long long)m);
  CO_CHECK(bed[0] == 0x6C && bed[1] == 0x1B && bed[2] == 0x01, COHERIT_E_SHAPE,
           "Not a valid SNP-major BED file");
  CO_CHECK(n_full < kMaxRows, COHERIT_E_SHAPE, "BED sample count %lld too large", (long long)n_full);
  const int64_t n = keep ? n_keep : n_full;
  if (keep)
    for (int64_t i = 0; i < n; ++i)
      CO_CHECK(keep[i] >= 0 && keep[i] < n_full, COHERIT_E_INDEX, "kept sample %lld out of range",
               (long long)i);
  coherit_sparse* h = new coherit_sparse();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = alloc_sparse(h, n, m, device);
  if (rc != COHERIT_OK) { free_sparse(h); return rc; }
  int64_t chunk_bytes = int64_t(256) << 20;
  if (const char* env = getenv("COHERIT_BED_CHUNK_BYTES")) {
    const long long v = atoll(env);
    if (v > 0) chunk_bytes = v;
  }
  const int64_t chunk = std::max<int64_t>(1, chunk_bytes / std::max<int64_t>(bps, 1));
  uint8_t* d_chunk = nullptr;
  int32_t* d_keep = nullptr;
  int32_t* d_nnz = nullptr;
  std::vector<int32_t> nnz_snp(static_cast<size_t>(std::max<int64_t>(m, 1)), 0);
  std::vector<int64_t> off(static_cast<size_t>(m + 1), 0);
  cudaError_t e = cudaSuccess;
  if (m > 0) {
    e = cudaMalloc(&d_chunk, static_cast<size_t>(std::min<int64_t>(chunk, m)) * bps);
    if (e == cudaSuccess) e = cudaMalloc(&d_nnz, sizeof(int32_t) * m);
    if (e == cudaSuccess && keep) {
      e = cudaMalloc(&d_keep, sizeof(int32_t) * std::max<int64_t>(n, 1));
      if (e == cudaSuccess && n > 0)
        e = cudaMemcpyAsync(d_keep, keep, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
    }
  }
  const uint8_t* body = bed + 3;
  // Pass 1: non-zero count of every SNP record.
  for (int64_t s_lo = 0; s_lo < m && e == cudaSuccess; s_lo += chunk) {
    const int64_t cnt = std::min<int64_t>(chunk, m - s_lo);
    e = cudaMemcpyAsync(d_chunk, body + s_lo * bps, static_cast<size_t>(cnt) * bps,
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) break;
    k_rec_count<<<blocks_for(cnt * 32, 256), 256, 0, st>>>(BedRecords{d_chunk, bps, d_keep},
                                                           cnt, n, d_nnz + s_lo); note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && m > 0)
    e = cudaMemcpyAsync(nnz_snp.data(), d_nnz, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) {
    for (int64_t j = 0; j < m; ++j) off[j + 1] = off[j] + nnz_snp[j];
    h->nnz = off[m];
    e = cudaMalloc(&h->d_entry, sizeof(uint32_t) * std::max<int64_t>(h->nnz, 1));
    if (e == cudaSuccess) h->device_bytes += sizeof(uint32_t) * std::max<int64_t>(h->nnz, 1);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->d_col_off, off.data(), sizeof(int64_t) * (m + 1),
                        cudaMemcpyHostToDevice, st);
  // Pass 2: entries in sample order.
  for (int64_t s_lo = 0; s_lo < m && e == cudaSuccess; s_lo += chunk) {
    const int64_t cnt = std::min<int64_t>(chunk, m - s_lo);
    e = cudaMemcpyAsync(d_chunk, body + s_lo * bps, static_cast<size_t>(cnt) * bps,
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) break;
    k_rec_fill<<<blocks_for(cnt * 32, 256), 256, 0, st>>>(BedRecords{d_chunk, bps, d_keep}, cnt,
                                                          n, h->d_col_off + s_lo, h->d_entry); note_launch();
    e = cudaGetLastError();
  }
  // The chunk buffer is reused by queued work until the stream drains.
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_chunk);
  cudaFree(d_keep);
  cudaFree(d_nnz);
  if (e != cudaSuccess) {
    free_sparse(h);
    return cuda_status(e, "sparse BED build");
  }
  rc = finish_sparse(h, st);
  if (rc != COHERIT_OK) { free_sparse(h); return rc; }
  *out = h;
  return COHERIT_OK;
}

int coherit_sparse_create_synthetic(int64_t n, int64_t m, uint64_t seed, uint32_t maf_lo_q24,
                                    uint32_t maf_hi_q24, uint32_t missing_q24, int device,
                                    void* stream, coherit_sparse_t** out) {
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "out handle pointer is NULL");
  *out = nullptr;
  CO_CHECK(maf_hi_q24 > maf_lo_q24 && maf_hi_q24 <= (1u << 23), COHERIT_E_SHAPE,
           "MAF range [%u, %u) / 2^24 must be non-empty and at most 0.5", maf_lo_q24, maf_hi_q24);
  coherit_sparse* h = new coherit_sparse();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = alloc_sparse(h, n, m, device);
  if (rc != COHERIT_OK) { free_sparse(h); return rc; }
  const SynthRecords src{seed, 0, maf_lo_q24, maf_hi_q24 - maf_lo_q24, missing_q24};
  int32_t* d_nnz = nullptr;
  std::vector<int32_t> nnz_snp(static_cast<size_t>(std::max<int64_t>(m, 1)), 0);
  std::vector<int64_t> off(static_cast<size_t>(m + 1), 0);
  cudaError_t e = cudaSuccess;
  if (m > 0) {
    e = cudaMalloc(&d_nnz, sizeof(int32_t) * m);
    if (e == cudaSuccess) {
      k_rec_count<<<blocks_for(m * 32, 256), 256, 0, st>>>(src, m, n, d_nnz); note_launch();
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(nnz_snp.data(), d_nnz, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e == cudaSuccess) {
    for (int64_t j = 0; j < m; ++j) off[j + 1] = off[j] + nnz_snp[j];
    h->nnz = off[m];
    e = cudaMalloc(&h->d_entry, sizeof(uint32_t) * std::max<int64_t>(h->nnz, 1));
    if (e == cudaSuccess) h->device_bytes += sizeof(uint32_t) * std::max<int64_t>(h->nnz, 1);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->d_col_off, off.data(), sizeof(int64_t) * (m + 1),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && m > 0) {
    k_rec_fill<<<blocks_for(m * 32, 256), 256, 0, st>>>(src, m, n, h->d_col_off, h->d_entry); note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_nnz);
  if (e != cudaSuccess) {
    free_sparse(h);
    return cuda_status(e, "synthetic sparse build");
  }
  rc = finish_sparse(h, st);
  if (rc != COHERIT_OK) { free_sparse(h); return rc; }
  *out = h;
  return COHERIT_OK;
}

int coherit_sparse_create_csc(int64_t n, int64_t m, const int64_t* col_off, const int32_t* rows,
                              const int8_t* vals, int device, void* stream,
                              coherit_sparse_t** out) {
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "out handle pointer is NULL");
  *out = nullptr;
  CO_CHECK(col_off != nullptr && m >= 0, COHERIT_E_SHAPE, "col_off is required");
  CO_CHECK(col_off[0] == 0, COHERIT_E_SHAPE, "col_off[0] must be 0");
  for (int64_t j = 0; j < m; ++j)
    CO_CHECK(col_off[j + 1] >= col_off[j], COHERIT_E_SHAPE, "col_off decreases at SNP %lld",
             (long long)j);
  const int64_t nnz = col_off[m];
  CO_CHECK(nnz == 0 || (rows != nullptr && vals != nullptr), COHERIT_E_SHAPE,
           "rows and vals are required for %lld entries", (long long)nnz);
  for (int64_t p = 0; p < nnz; ++p) {
    CO_CHECK(rows[p] >= 0 && rows[p] < n, COHERIT_E_INDEX, "entry %lld: sample %d out of range",
             (long long)p, rows[p]);
    CO_CHECK(vals[p] >= 1 && vals[p] <= 3, COHERIT_E_SHAPE,
             "entry %lld: value %d is not 1 (het), 2 (hom) or 3 (missing)", (long long)p,
             static_cast<int>(vals[p]));
  }
  coherit_sparse* h = new coherit_sparse();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = alloc_sparse(h, n, m, device);
  if (rc == COHERIT_OK) rc = upload_entries_from_host(h, col_off, rows, vals, st);
  if (rc == COHERIT_OK) rc = finish_sparse(h, st);
  if (rc != COHERIT_OK) { free_sparse(h); return rc; }
  *out = h;
  return COHERIT_OK;
}

int coherit_sparse_destroy(coherit_sparse_t* h) {
  if (h != nullptr) cudaSetDevice(h->device);
  free_sparse(h);
  return COHERIT_OK;
}

int coherit_sparse_info(const coherit_sparse_t* h, int64_t* n, int64_t* m, int64_t* nnz,
                        int64_t* n_missing, int64_t* device_bytes) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "sparse handle is NULL");
  if (n) *n = h->n;
  if (m) *m = h->m;
  if (nnz) *nnz = h->nnz;
  if (n_missing) {
    int64_t t = 0;
    for (int64_t v : h->n_miss) t += v;
    *n_missing = t;
  }
  if (device_bytes) *device_bytes = h->device_bytes;
  return COHERIT_OK;
}

int coherit_sparse_stats(const coherit_sparse_t* h, float* mean, float* inv, int64_t* n_het,
                         int64_t* n_hom, int64_t* n_miss, double* eff_m, double* mean_diag_atom) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "sparse handle is NULL");
  const size_t m = static_cast<size_t>(h->m);
  if (mean && m) std::memcpy(mean, h->mean.data(), sizeof(float) * m);
  if (inv && m) std::memcpy(inv, h->inv.data(), sizeof(float) * m);
  if (n_het && m) std::memcpy(n_het, h->n_het.data(), sizeof(int64_t) * m);
  if (n_hom && m) std::memcpy(n_hom, h->n_hom.data(), sizeof(int64_t) * m);
  if (n_miss && m) std::memcpy(n_miss, h->n_miss.data(), sizeof(int64_t) * m);
  if (eff_m) *eff_m = h->eff;
  if (mean_diag_atom) *mean_diag_atom = h->atom;
  return COHERIT_OK;
}

int coherit_sparse_set_stats(coherit_sparse_t* h, const float* mean, const float* inv,
                             void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "sparse handle is NULL");
  CO_CHECK(h->m == 0 || (mean != nullptr && inv != nullptr), COHERIT_E_SHAPE,
           "mean and inv are required");
  for (int64_t j = 0; j < h->m; ++j)
    CO_CHECK(std::isfinite(mean[j]) && std::isfinite(inv[j]) && inv[j] >= 0.f, COHERIT_E_SHAPE,
             "SNP %lld: mean and inverse sd must be finite, inverse sd >= 0", (long long)j);
  CO_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->m > 0) {
    std::memcpy(h->mean.data(), mean, sizeof(float) * h->m);
    std::memcpy(h->inv.data(), inv, sizeof(float) * h->m);
    CO_CUDA(cudaMemcpyAsync(h->d_mean, mean, sizeof(float) * h->m, cudaMemcpyHostToDevice, st));
    CO_CUDA(cudaMemcpyAsync(h->d_inv, inv, sizeof(float) * h->m, cudaMemcpyHostToDevice, st));
    CO_CUDA(cudaStreamSynchronize(st));
  }
  double eff = 0.0, mass = 0.0, base = 0.0;
  for (int64_t j = 0; j < h->m; ++j) {
    if (!(h->inv[j] > 0.f)) continue;
    eff += 1.0;
    mass += static_cast<double>(h->n - h->n_miss[j]);
    const float z0 = (0.f - h->mean[j]) * h->inv[j];
    base += static_cast<double>(z0) * static_cast<double>(z0);
  }
  h->eff = eff;
  h->atom = eff > 0.0 ? mass / (static_cast<double>(h->n) * eff) : 0.0;
  h->diag_base = base;
  return COHERIT_OK;
}

int coherit_sparse_read_csc(const coherit_sparse_t* h, int64_t* col_off, int32_t* rows,
                            int8_t* vals) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "sparse handle is NULL");
  CO_CUDA(cudaSetDevice(h->device));
  if (col_off)
    CO_CUDA(cudaMemcpy(col_off, h->d_col_off, sizeof(int64_t) * (h->m + 1), cudaMemcpyDeviceToHost));
  if ((rows || vals) && h->nnz > 0) {
    std::vector<uint32_t> e(static_cast<size_t>(h->nnz));
    CO_CUDA(cudaMemcpy(e.data(), h->d_entry, sizeof(uint32_t) * h->nnz, cudaMemcpyDeviceToHost));
    for (int64_t p = 0; p < h->nnz; ++p) {
      if (rows) rows[p] = static_cast<int32_t>(e[p] >> 2);
      if (vals) vals[p] = static_cast<int8_t>(e[p] & 3u);
    }
  }
  return COHERIT_OK;
}

int coherit_sparse_kv(coherit_sparse_t* h, const float* V, int64_t ldv, int32_t k, double scale,
                      float theta_e, float* out, int64_t ldo, void* stream) {
  return sparse_apply(h, true, V, ldv, k, scale, theta_e, out, ldo,
                      static_cast<cudaStream_t>(stream));
}

int coherit_sparse_xtv(coherit_sparse_t* h, const float* V, int64_t ldv, int32_t k, double scale,
                       float* out, int64_t ldo, void* stream) {
  return sparse_apply(h, false, V, ldv, k, scale, 0.f, out, ldo, static_cast<cudaStream_t>(stream));
}

int coherit_sparse_extract_columns(coherit_sparse_t* h, const int64_t* snp_idx, int32_t count,
                                   float* out, int64_t ldo, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "sparse handle is NULL");
  CO_CHECK(count >= 0 && ldo >= count, COHERIT_E_SHAPE, "bad count %d / ldo %lld", count,
           (long long)ldo);
  if (count == 0) return COHERIT_OK;
  CO_CHECK(snp_idx != nullptr && out != nullptr, COHERIT_E_SHAPE, "index and output are required");
  CO_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const dim3 blk(32, 8);
  const dim3 grd(static_cast<unsigned>((count + 31) / 32),
                 static_cast<unsigned>(std::min<int64_t>((h->n + 63) / 64, 4096)));
  k_extract_fill<<<grd, blk, 0, st>>>(out, ldo, h->n, count, snp_idx, h->m, h->d_mean, h->d_inv); note_launch();
  k_extract_scatter<<<blocks_for(int64_t(count) * 32, 256), 256, 0, st>>>(
      out, ldo, count, snp_idx, h->m, h->d_col_off, h->d_entry, h->d_mean, h->d_inv); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

int coherit_sparse_exact_diag(coherit_sparse_t* h, float* out, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "sparse handle is NULL");
  CO_CHECK(out != nullptr, COHERIT_E_SHAPE, "output is required");
  CO_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->d_diag == nullptr) {
    CO_CUDA(cudaMalloc(&h->d_diag, sizeof(double) * h->n));
    h->device_bytes += sizeof(double) * h->n;
  }
  CO_CUDA(cudaMemsetAsync(h->d_diag, 0, sizeof(double) * h->n, st));
  if (h->m > 0) {
    k_diag_entries<<<blocks_for(h->m * 32, 256), 256, 0, st>>>(
        h->d_col_off, h->d_entry, h->m, h->d_mean, h->d_inv, h->d_diag); note_launch();
  }
  k_diag_finish<<<blocks_for(h->n, 256), 256, 0, st>>>(h->d_diag, h->n,
                                                                         h->diag_base, h->eff, out); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

}  // extern "C"
