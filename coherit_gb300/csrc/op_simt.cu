// op_simt.cu -- the plain FP32 form of the genotype operator on CUDA cores.
//
// This is the reference arithmetic of kv_impl.py:69-113 without tensor cores:
// every genotype is decoded to diff = (g - mean) in FP32 (0 where missing,
// i.e. mean-imputed), then T = diff^T V and out = diff (w * T) are FP32 FMA
// contractions.  It serves as the "plain FP32 single-fit GPU path" and as an
// independent check of the tensor-core path.  One request (column group) per
// launch.
#include <algorithm>
#include <cstring>

#include "coherit_internal.cuh"

namespace coherit {

constexpr int kSimtCols = 32;  // columns per CTA
constexpr int kSimtRows = 64;  // slots (K1) or samples (K2) per CTA

struct SimtParams {
  int64_t n, n_pad, m_pad, n_chunks, n_panels;
  int k, kp, stacked, xtv, use_theta_e;
  int64_t ldv, ldo;
  const uint8_t* geno_t;
  const uint8_t* geno_s;
  const float* mean;
  const float* inv;
  const uint8_t* mask;
  const int32_t* comp_of_slot;
  const int32_t* snp_of_slot;
  const int64_t* comp_slot_start;
  const float* snpw;
  float cscale[64];
  float theta_e;
  const float* V;
  float* sf;    // m_pad x kp
  float* out;   // K2 output or X^T V output
};

// T block rows -> diff[sample r][slot jj] in shared memory.
__global__ void __launch_bounds__(256) k_simt_k1(const __grid_constant__ SimtParams p) {
  __shared__ float D[kPanel][kSimtRows + 1];
  __shared__ float Vs[kPanel][kSimtCols];
  const int t = threadIdx.x;
  const int64_t slot0 = static_cast<int64_t>(blockIdx.x) * kSimtRows;
  const int c0 = blockIdx.y * kSimtCols;
  const int64_t tt = slot0 / kTile;
  const int rbase = static_cast<int>(slot0 % kTile);
  const int jj = t % kSimtRows;
  const int cg = t / kSimtRows;  // 0..3 -> 8 columns each
  float acc[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) acc[u] = 0.f;
  // decode role: 4 threads per slot row, one 32-bit word (16 samples) each
  const int drow = t / 4, dword = t % 4;
  const float mu = p.mean[slot0 + drow];
  for (int64_t q = 0; q < p.n_chunks; ++q) {
    const uint32_t w = reinterpret_cast<const uint32_t*>(
        p.geno_t + ((tt * p.n_chunks + q) * kTile + rbase + drow) * kRowBytes)[dword];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int e = dword * 16 + r;
      const uint32_t code = (w >> row_shift(e)) & 3u;
      D[e][drow] = code == 3u ? 0.f : (static_cast<float>(code) - mu);
    }
    for (int idx = t; idx < kPanel * kSimtCols; idx += 256) {
      const int r = idx / kSimtCols, c = idx % kSimtCols;
      const int64_t i = q * kPanel + r;
      float v = 0.f;
      if (i < p.n && c0 + c < p.k && (p.mask == nullptr || p.mask[i] != 0))
        v = p.V[i * p.ldv + c0 + c];
      Vs[r][c] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < kPanel; ++r) {
      const float d = D[r][jj];
#pragma unroll
      for (int u = 0; u < 8; ++u) acc[u] = fmaf(d, Vs[r][cg * 8 + u], acc[u]);
    }
    __syncthreads();
  }
  const int64_t j = slot0 + jj;
  const int32_t snp = p.snp_of_slot[j];
  const float iv = p.inv[j];
  float w = (p.xtv ? iv : iv * iv) * p.cscale[p.comp_of_slot[j]];
  if (p.snpw != nullptr) w *= snp >= 0 ? p.snpw[snp] : 0.f;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int c = c0 + cg * 8 + u;
    if (c >= p.kp) continue;
    const float s = (c < p.k) ? w * acc[u] : 0.f;
    if (p.xtv) {
      if (snp >= 0 && c < p.k) p.out[static_cast<int64_t>(snp) * p.ldo + c] = s;
    } else {
      p.sf[j * p.kp + c] = s;
    }
  }
}

__global__ void __launch_bounds__(256) k_simt_k2(const __grid_constant__ SimtParams p) {
  __shared__ float D[kPanel][kSimtRows + 1];  // [slot jj][sample r]
  __shared__ float Ss[kPanel][kSimtCols];
  __shared__ float mus[kPanel];
  const int t = threadIdx.x;
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * kSimtRows;
  const int c0 = blockIdx.y * kSimtCols;
  const int comp = blockIdx.z;
  const int64_t st = i0 / kTile;
  const int rbase = static_cast<int>(i0 % kTile);
  int64_t p0 = 0, p1 = p.n_panels;
  if (p.stacked) {
    p0 = p.comp_slot_start[comp] / kPanel;
    p1 = p.comp_slot_start[comp + 1] / kPanel;
  }
  const int r_own = t % kSimtRows;
  const int cg = t / kSimtRows;
  float acc[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) acc[u] = 0.f;
  const int drow = t / 4, dword = t % 4;
  for (int64_t pn = p0; pn < p1; ++pn) {
    if (t < kPanel) mus[t] = p.mean[pn * kPanel + t];
    __syncthreads();
    const uint32_t w = reinterpret_cast<const uint32_t*>(
        p.geno_s + ((st * p.n_panels + pn) * kTile + rbase + drow) * kRowBytes)[dword];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int e = dword * 16 + r;
      const uint32_t code = (w >> row_shift(e)) & 3u;
      D[e][drow] = code == 3u ? 0.f : (static_cast<float>(code) - mus[e]);
    }
    for (int idx = t; idx < kPanel * kSimtCols; idx += 256) {
      const int r = idx / kSimtCols, c = idx % kSimtCols;
      Ss[r][c] = (c0 + c < p.kp) ? p.sf[(pn * kPanel + r) * p.kp + c0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int e = 0; e < kPanel; ++e) {
      const float d = D[e][r_own];
#pragma unroll
      for (int u = 0; u < 8; ++u) acc[u] = fmaf(d, Ss[e][cg * 8 + u], acc[u]);
    }
    __syncthreads();
  }
  const int64_t i = i0 + r_own;
  if (i >= p.n) return;
  const bool keep = p.mask == nullptr || p.mask[i] != 0;
  float* outb = p.out + static_cast<int64_t>(p.stacked ? comp : 0) * p.n * p.ldo;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int c = c0 + cg * 8 + u;
    if (c >= p.k) continue;
    float v = acc[u];
    if (p.use_theta_e) v += p.theta_e * p.V[i * p.ldv + c];
    outb[i * p.ldo + c] = keep ? v : 0.f;
  }
}

// b (m x C) -> sf = inv_sd * b for Z b.
__global__ void k_simt_prep_b(const __grid_constant__ SimtParams p, const float* __restrict__ b,
                              int64_t ldb) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j >= p.m_pad) return;
  const int32_t snp = p.snp_of_slot[j];
  for (int c = 0; c < p.kp; ++c) {
    float s = 0.f;
    if (snp >= 0 && c < p.k) s = p.inv[j] * b[static_cast<int64_t>(snp) * ldb + c];
    p.sf[j * p.kp + c] = s;
  }
}

int run_operator_fp32(coherit_geno* h, const OpDesc& d, cudaStream_t st) {
  CO_CHECK(d.n_groups == 1, COHERIT_E_UNSUPPORTED,
           "the FP32 operator form serves one request per launch");
  CO_CHECK(h->G <= 64, COHERIT_E_UNSUPPORTED, "the FP32 operator form supports <= 64 components");
  const int kp = static_cast<int>(round_up(std::max(d.k, 1), 16));
  int rc = ensure_ws_bytes(h, static_cast<size_t>(h->m_pad) * kp * sizeof(float));
  if (rc != COHERIT_OK) return rc;
  const int slot = d.slot_of_group[0];
  CO_CHECK(slot >= 0 && slot < static_cast<int>(h->slots.size()) && h->slots[slot].used,
           COHERIT_E_INDEX, "stats slot %d is not initialised", slot);
  const StatsSlot& s = h->slots[slot];
  SimtParams p;
  memset(&p, 0, sizeof(p));
  p.n = h->n;
  p.n_pad = h->n_pad;
  p.m_pad = h->m_pad;
  p.n_chunks = h->n_chunks;
  p.n_panels = h->n_panels;
  p.k = d.k;
  p.kp = kp;
  p.stacked = d.mode == COHERIT_MODE_STACKED ? 1 : 0;
  p.xtv = d.xtv ? 1 : 0;
  p.use_theta_e = d.theta_e.empty() ? 0 : 1;
  p.theta_e = d.theta_e.empty() ? 0.f : d.theta_e[0];
  p.ldv = d.ldv;
  p.ldo = d.ldo;
  p.geno_t = h->geno_t;
  p.geno_s = h->geno_s;
  p.mean = s.mean;
  p.inv = s.inv;
  p.mask = s.row_mask;
  p.comp_of_slot = h->d_comp_of_slot;
  p.snp_of_slot = h->d_snp_of_slot;
  p.comp_slot_start = h->d_comp_slot_start;
  p.snpw = d.snp_weight;
  for (int g = 0; g < h->G; ++g) p.cscale[g] = d.comp_scale[g];
  p.V = d.V;
  p.out = d.out;
  // S in FP32 (m_pad x kp) at the start of the workspace.
  p.sf = static_cast<float*>(h->ws.base);
  const unsigned cblocks = static_cast<unsigned>((kp + kSimtCols - 1) / kSimtCols);
  if (d.zxb) {
    k_simt_prep_b<<<static_cast<unsigned>((h->m_pad + 127) / 128), 128, 0, st>>>(p, d.V, d.ldv); note_launch();
    p.use_theta_e = 0;
  } else {
    k_simt_k1<<<dim3(static_cast<unsigned>(h->m_pad / kSimtRows), cblocks), 256, 0, st>>>(p); note_launch();
  }
  CO_CUDA(cudaGetLastError());
  if (d.xtv) return COHERIT_OK;
  const unsigned nz = p.stacked ? static_cast<unsigned>(h->G) : 1u;
  k_simt_k2<<<dim3(static_cast<unsigned>(h->n_pad / kSimtRows), cblocks, nz), 256, 0, st>>>(p); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

}  // namespace coherit
