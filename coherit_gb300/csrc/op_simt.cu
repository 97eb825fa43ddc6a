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
#include <type_traits>

#include "coherit_internal.cuh"

namespace coherit {

// Tiles: COLS right-hand-side columns (8, 16 or 32, the narrowest that
// holds the block's columns in few launches) x ROWS = 2048 / COLS slots (K1)
// or samples (K2) per CTA of 256 threads; every thread owns one row and 8
// columns.  Narrow PCG blocks then do no work for padding columns.
constexpr int kSimtOut = 2048;  // outputs per CTA

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

template <int COLS>
constexpr int simt_rows() { return kSimtOut / COLS; }
template <int COLS>
constexpr size_t simt_smem() {
  return sizeof(float) * (static_cast<size_t>(kPanel) * (simt_rows<COLS>() + 1) + kPanel * COLS +
                          kPanel);
}

// K1: T = diff^T V for ROWS slots; the T block rows of a chunk are decoded to
// diff[sample][slot] in shared memory (4 threads per slot row, one 32-bit
// word = 16 samples each).
template <int COLS>
__global__ void __launch_bounds__(256) k_simt_k1(const __grid_constant__ SimtParams p) {
  constexpr int ROWS = simt_rows<COLS>();
  extern __shared__ float sm[];
  float* D = sm;                               // [64][ROWS + 1]
  float* Vs = sm + kPanel * (ROWS + 1);        // [64][COLS]
  const int t = threadIdx.x;
  const int64_t slot0 = static_cast<int64_t>(blockIdx.x) * ROWS;
  const int c0 = blockIdx.y * COLS;
  const int jj = t % ROWS;
  const int cg = t / ROWS;  // column group of 8
  float acc[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) acc[u] = 0.f;
  constexpr int kWords = 4 * ROWS / 256;  // decode words per thread and chunk
  float mu[kWords];
  const uint8_t* rowp[kWords];
#pragma unroll
  for (int x = 0; x < kWords; ++x) {
    const int widx = t + 256 * x;
    const int64_t slot = slot0 + widx / 4;
    mu[x] = p.mean[slot];
    rowp[x] = p.geno_t + ((slot / kTile) * p.n_chunks * kTile + slot % kTile) * kRowBytes +
              4 * (widx % 4);
  }
  for (int64_t q = 0; q < p.n_chunks; ++q) {
#pragma unroll
    for (int x = 0; x < kWords; ++x) {
      const int widx = t + 256 * x;
      const int drow = widx / 4, dword = widx % 4;
      const uint32_t w = *reinterpret_cast<const uint32_t*>(rowp[x] + q * kTile * kRowBytes);
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const int e = dword * 16 + r;
        const uint32_t code = (w >> row_shift(e)) & 3u;
        D[e * (ROWS + 1) + drow] = code == 3u ? 0.f : (static_cast<float>(code) - mu[x]);
      }
    }
    for (int idx = t; idx < kPanel * COLS; idx += 256) {
      const int r = idx / COLS, c = idx % COLS;
      const int64_t i = q * kPanel + r;
      float v = 0.f;
      if (i < p.n && c0 + c < p.k && (p.mask == nullptr || p.mask[i] != 0))
        v = p.V[i * p.ldv + c0 + c];
      Vs[r * COLS + c] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int r = 0; r < kPanel; ++r) {
      const float d = D[r * (ROWS + 1) + jj];
#pragma unroll
      for (int u = 0; u < 8; ++u) acc[u] = fmaf(d, Vs[r * COLS + cg * 8 + u], acc[u]);
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

// K2: out = diff S for ROWS samples; the S block rows of a panel are decoded
// to diff[slot][sample] in shared memory.
template <int COLS>
__global__ void __launch_bounds__(256) k_simt_k2(const __grid_constant__ SimtParams p) {
  constexpr int ROWS = simt_rows<COLS>();
  extern __shared__ float sm[];
  float* D = sm;                          // [64 slots][ROWS + 1]
  float* Ss = sm + kPanel * (ROWS + 1);   // [64][COLS]
  float* mus = Ss + kPanel * COLS;        // [64]
  const int t = threadIdx.x;
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * ROWS;
  const int c0 = blockIdx.y * COLS;
  const int comp = blockIdx.z;
  int64_t p0 = 0, p1 = p.n_panels;
  if (p.stacked) {
    p0 = p.comp_slot_start[comp] / kPanel;
    p1 = p.comp_slot_start[comp + 1] / kPanel;
  }
  const int r_own = t % ROWS;
  const int cg = t / ROWS;
  float acc[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) acc[u] = 0.f;
  constexpr int kWords = 4 * ROWS / 256;
  const uint8_t* rowp[kWords];
#pragma unroll
  for (int x = 0; x < kWords; ++x) {
    const int widx = t + 256 * x;
    const int64_t i = i0 + widx / 4;
    rowp[x] = p.geno_s + ((i / kTile) * p.n_panels * kTile + i % kTile) * kRowBytes +
              4 * (widx % 4);
  }
  for (int64_t pn = p0; pn < p1; ++pn) {
    if (t < kPanel) mus[t] = p.mean[pn * kPanel + t];
    __syncthreads();
#pragma unroll
    for (int x = 0; x < kWords; ++x) {
      const int widx = t + 256 * x;
      const int drow = widx / 4, dword = widx % 4;
      const uint32_t w = *reinterpret_cast<const uint32_t*>(rowp[x] + pn * kTile * kRowBytes);
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const int e = dword * 16 + r;
        const uint32_t code = (w >> row_shift(e)) & 3u;
        D[e * (ROWS + 1) + drow] = code == 3u ? 0.f : (static_cast<float>(code) - mus[e]);
      }
    }
    for (int idx = t; idx < kPanel * COLS; idx += 256) {
      const int r = idx / COLS, c = idx % COLS;
      Ss[r * COLS + c] = (c0 + c < p.kp) ? p.sf[(pn * kPanel + r) * p.kp + c0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int e = 0; e < kPanel; ++e) {
      const float d = D[e * (ROWS + 1) + r_own];
#pragma unroll
      for (int u = 0; u < 8; ++u) acc[u] = fmaf(d, Ss[e * COLS + cg * 8 + u], acc[u]);
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
  if (d.zxb) {
    k_simt_prep_b<<<static_cast<unsigned>((h->m_pad + 127) / 128), 128, 0, st>>>(p, d.V, d.ldv); note_launch();
    p.use_theta_e = 0;
    CO_CUDA(cudaGetLastError());
  }
  // Narrowest tile that holds the block (kp is a multiple of 16; 8 only for
  // one-column blocks padded to 16 would waste half the CTA).
  const int cols = kp <= 16 ? 16 : 32;
  auto run = [&](auto cols_tag) -> int {
    constexpr int COLS = decltype(cols_tag)::value;
    constexpr int ROWS = simt_rows<COLS>();
    const unsigned cblocks = static_cast<unsigned>((kp + COLS - 1) / COLS);
    const size_t smem = simt_smem<COLS>();
    if (!d.zxb) {
      CO_CUDA(cudaFuncSetAttribute(k_simt_k1<COLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(smem)));
      k_simt_k1<COLS><<<dim3(static_cast<unsigned>(h->m_pad / ROWS), cblocks), 256, smem, st>>>(p);
      note_launch();
      CO_CUDA(cudaGetLastError());
    }
    if (d.xtv) return COHERIT_OK;
    const unsigned nz = p.stacked ? static_cast<unsigned>(h->G) : 1u;
    CO_CUDA(cudaFuncSetAttribute(k_simt_k2<COLS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)));
    k_simt_k2<COLS><<<dim3(static_cast<unsigned>(h->n_pad / ROWS), cblocks, nz), 256, smem, st>>>(p);
    note_launch();
    CO_CUDA(cudaGetLastError());
    return COHERIT_OK;
  };
  if (cols == 16) return run(std::integral_constant<int, 16>());
  return run(std::integral_constant<int, 32>());
}

}  // namespace coherit
