// lowrank.cu -- the projected-core preconditioner's per-iteration apply
//     out = a V + U (G (U^T V))
// (precond.py:42-84: M^{-1} v with G = (dI + C)^{-1} - d^{-1} I and a = 1/d,
// or M^{-1/2} v with G = Q diag(e^{-1/2}) Q^T - d^{-1/2} I and a = d^{-1/2})
// for a tall orthonormal basis U (n x r, row-major) and a block V (n x k).
//
// Three launches: the two n-long contractions are register-tiled FP32
// CUDA-core GEMMs (64 x 64 output tiles, 4 x 4 per thread, 16-deep shared
// stages), the r x r product in between sums the per-slice partials of
// U^T V and applies G.  Work per apply: 4 n r k flops, 4 n r bytes of U read
// twice; at n = 100,000, r = 256, k = 12 about 25 us of HBM time.
#include "coherit_internal.cuh"

namespace coherit {
namespace {

constexpr int kT = 64;      // output tile edge
constexpr int kDepth = 16;  // contraction depth per shared stage
constexpr int kRowsPerSlice = 2048;

// part[s] (r x k) = U[rows of slice s]^T V[rows of slice s].  Grid:
// (ceil(r / 64), ceil(k / 64), slices).  Thread (ty, tx) owns rows
// 4 ty..4 ty + 3 of the tile's r range and columns 4 tx..4 tx + 3.
__global__ void __launch_bounds__(256) k_lr_utv(int64_t n, int r, int k,
                                                const float* __restrict__ U, int64_t ldu,
                                                const float* __restrict__ V, int64_t ldv,
                                                float* __restrict__ part) {
  __shared__ float Us[kDepth][kT];
  __shared__ float Vs[kDepth][kT];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.x * kT, c0 = blockIdx.y * kT;
  const int64_t r0 = static_cast<int64_t>(blockIdx.z) * kRowsPerSlice;
  const int64_t r1 = min(n, r0 + kRowsPerSlice);
  float acc[4][4] = {};
  for (int64_t base = r0; base < r1; base += kDepth) {
    // 16 rows x 64 entries of U and of V: 1,024 floats each, 4 per thread.
    for (int e = threadIdx.x; e < kDepth * kT; e += 256) {
      const int rr = e / kT, cc = e % kT;
      const int64_t row = base + rr;
      Us[rr][cc] = (row < r1 && i0 + cc < r) ? U[row * ldu + i0 + cc] : 0.f;
      Vs[rr][cc] = (row < r1 && c0 + cc < k) ? V[row * ldv + c0 + cc] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int rr = 0; rr < kDepth; ++rr) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = Us[rr][4 * ty + q];
        b[q] = Vs[rr][4 * tx + q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
  float* out = part + static_cast<int64_t>(blockIdx.z) * r * k;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int i = i0 + 4 * ty + p;
    if (i >= r) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + 4 * tx + q;
      if (c < k) out[static_cast<int64_t>(i) * k + c] = acc[p][q];
    }
  }
}

// Y (r x k) = G (r x r, row-major) * W, W = sum over slices of part (the
// slice sums in FP64).  One thread per (i, c); W is summed into shared
// memory per column block first.
__global__ void __launch_bounds__(256) k_lr_mid(int r, int k, int slices,
                                                const float* __restrict__ part,
                                                const float* __restrict__ G, int64_t ldg,
                                                float* __restrict__ Y) {
  extern __shared__ float Ws[];  // r x 8 columns of W
  const int c0 = blockIdx.x * 8;
  const int cw = min(8, k - c0);
  for (int e = threadIdx.x; e < r * cw; e += blockDim.x) {
    const int l = e / cw, cc = e % cw;
    double s = 0.0;
    for (int z = 0; z < slices; ++z)
      s += static_cast<double>(part[(static_cast<int64_t>(z) * r + l) * k + c0 + cc]);
    Ws[l * 8 + cc] = static_cast<float>(s);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < r * cw; e += blockDim.x) {
    const int i = e / cw, cc = e % cw;
    float s = 0.f;
    for (int l = 0; l < r; ++l) s = fmaf(G[static_cast<int64_t>(i) * ldg + l], Ws[l * 8 + cc], s);
    Y[static_cast<int64_t>(i) * k + c0 + cc] = s;
  }
}

// out (n x k) = a V + U Y.  Grid: (ceil(n / 64), ceil(k / 64)).
__global__ void __launch_bounds__(256) k_lr_expand(int64_t n, int r, int k, float a,
                                                   const float* __restrict__ U, int64_t ldu,
                                                   const float* __restrict__ Y,
                                                   const float* __restrict__ V, int64_t ldv,
                                                   float* __restrict__ out, int64_t ldo) {
  __shared__ float Us[kT][kDepth + 1];
  __shared__ float Ys[kDepth][kT];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t row0 = static_cast<int64_t>(blockIdx.x) * kT;
  const int c0 = blockIdx.y * kT;
  float acc[4][4] = {};
  for (int l0 = 0; l0 < r; l0 += kDepth) {
    for (int e = threadIdx.x; e < kT * kDepth; e += 256) {
      const int rr = e / kDepth, ll = e % kDepth;
      const int64_t row = row0 + rr;
      Us[rr][ll] = (row < n && l0 + ll < r) ? U[row * ldu + l0 + ll] : 0.f;
    }
    for (int e = threadIdx.x; e < kDepth * kT; e += 256) {
      const int ll = e / kT, cc = e % kT;
      Ys[ll][cc] = (l0 + ll < r && c0 + cc < k) ? Y[static_cast<int64_t>(l0 + ll) * k + c0 + cc]
                                                 : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int ll = 0; ll < kDepth; ++ll) {
      float u[4], y[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        u[q] = Us[4 * ty + q][ll];
        y[q] = Ys[ll][4 * tx + q];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(u[p], y[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int64_t row = row0 + 4 * ty + p;
    if (row >= n) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + 4 * tx + q;
      if (c < k) out[row * ldo + c] = fmaf(a, V[row * ldv + c], acc[p][q]);
    }
  }
}

}  // namespace
}  // namespace coherit

using namespace coherit;

extern "C" int coherit_lowrank_workspace_floats(int64_t n, int32_t r, int32_t k, int64_t* floats) {
  CO_CHECK(n >= 1 && r >= 1 && k >= 1 && floats != nullptr, COHERIT_E_SHAPE,
           "low-rank apply needs n, r, k >= 1");
  const int64_t slices = (n + kRowsPerSlice - 1) / kRowsPerSlice;
  *floats = (slices + 1) * static_cast<int64_t>(r) * k;
  return COHERIT_OK;
}

extern "C" int coherit_lowrank_apply(int64_t n, int32_t r, int32_t k, const float* U, int64_t ldu,
                                     const float* G, int64_t ldg, float a, const float* V,
                                     int64_t ldv, float* out, int64_t ldo, float* work,
                                     int64_t work_floats, void* stream) {
  CO_CHECK(n >= 1 && r >= 1 && k >= 1, COHERIT_E_SHAPE, "low-rank apply needs n, r, k >= 1");
  CO_CHECK(ldu >= r && ldg >= r && ldv >= k && ldo >= k, COHERIT_E_SHAPE,
           "row strides must be at least the row lengths");
  CO_CHECK(U && G && V && out && work, COHERIT_E_SHAPE, "null pointer");
  CO_CHECK(r <= 4096, COHERIT_E_SHAPE, "rank %d exceeds 4096", r);
  const int64_t slices = (n + kRowsPerSlice - 1) / kRowsPerSlice;
  CO_CHECK(slices <= 65535, COHERIT_E_SHAPE, "n too large for one launch");
  CO_CHECK(work_floats >= (slices + 1) * static_cast<int64_t>(r) * k, COHERIT_E_SHAPE,
           "workspace holds %lld floats, needs %lld", static_cast<long long>(work_floats),
           static_cast<long long>((slices + 1) * static_cast<int64_t>(r) * k));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float* part = work;
  float* Y = work + slices * static_cast<int64_t>(r) * k;
  const unsigned tiles_r = static_cast<unsigned>((r + kT - 1) / kT);
  const unsigned tiles_k = static_cast<unsigned>((k + kT - 1) / kT);
  k_lr_utv<<<dim3(tiles_r, tiles_k, static_cast<unsigned>(slices)), 256, 0, st>>>(n, r, k, U, ldu,
                                                                                  V, ldv, part);
  note_launch();
  const size_t mid_smem = static_cast<size_t>(r) * 8 * sizeof(float);
  if (mid_smem > 48 * 1024)
    CO_CUDA(cudaFuncSetAttribute(k_lr_mid, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(mid_smem)));
  k_lr_mid<<<static_cast<unsigned>((k + 7) / 8), 256, mid_smem, st>>>(
      r, k, static_cast<int>(slices), part, G, ldg, Y);
  note_launch();
  k_lr_expand<<<dim3(static_cast<unsigned>((n + kT - 1) / kT), tiles_k), 256, 0, st>>>(
      n, r, k, a, U, ldu, Y, V, ldv, out, ldo);
  note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}
