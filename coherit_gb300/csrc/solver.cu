// solver.cu -- block-PCG vector kernels (column reductions in FP64, fused
// state and direction updates; pcg.py:31-65) and the tensor-core self-test
// that checks the MMA operand layouts on one tile.
#include <cmath>
#include <cstring>

#include "coherit_internal.cuh"
#include "tc_ptx.cuh"

namespace coherit {

constexpr int kRedThreads = 256;
constexpr int kRedCols = 32;  // columns per CTA in the reductions

// Column reduction: each CTA owns up to 32 columns and a strided set of rows;
// warp-shuffle partial sums are combined with FP64 atomics.
__global__ void k_colreduce(int op, int64_t n, int k, const float* __restrict__ A, int64_t lda,
                            const float* __restrict__ B, int64_t ldb, double* __restrict__ out) {
  __shared__ double part[kRedThreads / 32][kRedCols];
  const int c0 = blockIdx.y * kRedCols;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = c0 + lane;
  double s = 0.0;
  if (c < k) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(kRedThreads / 32) + warp; i < n;
         i += static_cast<int64_t>(gridDim.x) * (kRedThreads / 32)) {
      const float a = A[i * lda + c];
      const float b = op == 0 ? B[i * ldb + c] : a;
      s += static_cast<double>(a) * static_cast<double>(b);
    }
  }
  part[warp][lane] = s;
  __syncthreads();
  if (warp == 0 && c < k) {
    double t = 0.0;
    for (int w = 0; w < kRedThreads / 32; ++w) t += part[w][lane];
    atomicAdd(&out[c], t);
  }
}

__global__ void k_pcg_state(int64_t n, int k, float* __restrict__ X, int64_t ldx,
                            float* __restrict__ R, int64_t ldr, const float* __restrict__ P,
                            int64_t ldp, const float* __restrict__ AP, int64_t ldap,
                            const double* __restrict__ rs, const double* __restrict__ denom,
                            const uint8_t* __restrict__ active, int32_t* __restrict__ breakdown) {
  extern __shared__ float alpha_s[];
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    const double r = rs[c], d = denom[c];
    const bool valid = r > 0.0 && d > 0.0 && isfinite(r) && isfinite(d);
    const bool moving = active[c] != 0 && valid;
    alpha_s[c] = moving ? static_cast<float>(r / d) : 0.f;
    if (blockIdx.x == 0 && active[c] != 0 && !valid) atomicOr(breakdown, 1);
  }
  __syncthreads();
  const int64_t total = n * k;
  for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
       idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t i = idx / k;
    const int c = static_cast<int>(idx % k);
    const float a = alpha_s[c];
    X[i * ldx + c] = X[i * ldx + c] + P[i * ldp + c] * a;
    R[i * ldr + c] = R[i * ldr + c] - AP[i * ldap + c] * a;
  }
}

__global__ void k_pcg_dir(int64_t n, int k, float* __restrict__ P, int64_t ldp,
                          const float* __restrict__ Z, int64_t ldz, const double* __restrict__ rs_new,
                          const double* __restrict__ rnorm2, const double* __restrict__ rs_old,
                          const double* __restrict__ thr) {
  extern __shared__ float beta_s[];  // k betas then k active flags
  float* act_s = beta_s + k;
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    const bool act = sqrt(rnorm2[c]) > thr[c];
    const double ro = rs_old[c] > 0.0 ? rs_old[c] : 1.0;
    beta_s[c] = act ? static_cast<float>(rs_new[c] / ro) : 0.f;
    act_s[c] = act ? 1.f : 0.f;
  }
  __syncthreads();
  const int64_t total = n * k;
  for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
       idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t i = idx / k;
    const int c = static_cast<int>(idx % k);
    P[i * ldp + c] = act_s[c] != 0.f ? Z[i * ldz + c] + P[i * ldp + c] * beta_s[c] : 0.f;
  }
}

__global__ void k_pcg_dir_scalars(int k, const double* __restrict__ rs_new,
                                  const double* __restrict__ rnorm2, double* __restrict__ rs_old,
                                  const double* __restrict__ thr, uint8_t* __restrict__ active,
                                  double* __restrict__ rnorm_out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const double rn = sqrt(rnorm2[c]);
  const bool act = rn > thr[c];
  active[c] = act ? 1 : 0;
  rs_old[c] = act ? rs_new[c] : 0.0;
  rnorm_out[c] = rn;
}

static unsigned elem_grid(int64_t total) {
  int64_t g = (total + 255) / 256;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  return static_cast<unsigned>(g);
}

// ----------------------------------------------------- tensor-core self-test
// One CTA of 128 threads computes D(128x16) = A(128x16) B(16x16)^T with
// small exact integers.  variant 0: A from tensor memory (tcgen05.st), B
// from shared memory; variant 1: both from shared memory.  Both operands use
// the K-major, no-swizzle core-matrix layout of the operator kernels.
__host__ __device__ inline int probe_a(int m, int k) { return ((m * 3 + k * 5) % 7) - 3; }
__host__ __device__ inline int probe_b(int n, int k) { return ((n * 2 + k) % 5) - 2; }

__global__ void __launch_bounds__(128, 1) k_probe_mma(int variant, float* __restrict__ out,
                                                      int* __restrict__ err) {
  __shared__ __align__(1024) __nv_bfloat16 a_s[128 * 16];
  __shared__ __align__(1024) __nv_bfloat16 b_s[16 * 16];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ int abort_flag;
  const int t = threadIdx.x;
  const int warp = t >> 5;
  // B: 16 (N) x 16 (K), core matrix (n/8, k/8) at ((n/8)*2 + k/8)*64 elements.
  for (int idx = t; idx < 256; idx += 128) {
    const int n = idx / 16, k = idx % 16;
    b_s[((n >> 3) * 2 + (k >> 3)) * 64 + (n & 7) * 8 + (k & 7)] =
        __float2bfloat16_rn(static_cast<float>(probe_b(n, k)));
  }
  for (int k = 0; k < 16; ++k) {
    a_s[((t >> 3) * 2 + (k >> 3)) * 64 + (t & 7) * 8 + (k & 7)] =
        __float2bfloat16_rn(static_cast<float>(probe_a(t, k)));
  }
  if (t == 0) {
    ptx::mbar_init(&bar, 1);
    abort_flag = 0;
    ptx::fence_barrier_init();
  }
  ptx::fence_proxy_async_smem();
  if (warp == 0) ptx::tmem_alloc(&tslot, 64);
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = tslot;
  const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
  if (variant == 0) {
    uint32_t a[32];
    for (int j = 0; j < 32; ++j) a[j] = 0u;
    for (int j = 0; j < 8; ++j) {
      const __nv_bfloat16 lo = __float2bfloat16_rn(static_cast<float>(probe_a(t, 2 * j)));
      const __nv_bfloat16 hi = __float2bfloat16_rn(static_cast<float>(probe_a(t, 2 * j + 1)));
      a[j] = static_cast<uint32_t>(__bfloat16_as_ushort(lo)) |
             (static_cast<uint32_t>(__bfloat16_as_ushort(hi)) << 16);
    }
    ptx::tmem_st32(tmem + lane_base + 32u, a);
    ptx::tmem_wait_st();
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (t == 0) {
    ptx::tc_fence_after();
    const uint32_t idesc = ptx::idesc_bf16_f32(128, 16);
    const uint64_t bd = ptx::smem_desc(ptx::smem_addr(b_s), 128u, 256u);
    if (variant == 0) {
      ptx::mma_ts(tmem, tmem + 32u, bd, idesc, 0u);
    } else {
      const uint64_t ad = ptx::smem_desc(ptx::smem_addr(a_s), 128u, 256u);
      ptx::mma_ss(tmem, ad, bd, idesc, 0u);
    }
    ptx::mma_commit(&bar);
  }
  const bool ok = ptx::mbar_wait(&bar, 0, err, 21, &abort_flag);
  if (__all_sync(0xffffffffu, ok)) {
    ptx::tc_fence_after();
    uint32_t r[16];
    ptx::tmem_ld16(tmem + lane_base, r);
    ptx::tmem_wait_ld();
    for (int j = 0; j < 16; ++j) out[t * 16 + j] = __uint_as_float(r[j]);
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 64);
  }
}

}  // namespace coherit

using namespace coherit;

extern "C" {

int coherit_colreduce(int32_t op, int64_t n, int32_t k, const float* A, int64_t lda,
                      const float* B, int64_t ldb, double* out, void* stream) {
  CO_CHECK(op == 0 || op == 1, COHERIT_E_SHAPE, "unknown reduction %d", op);
  CO_CHECK(k >= 0 && n >= 0, COHERIT_E_SHAPE, "negative extents");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (k == 0) return COHERIT_OK;
  CO_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * k, st));
  if (n == 0) return COHERIT_OK;
  int64_t gx = (n + 63) / 64;
  if (gx > 1024) gx = 1024;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>((k + kRedCols - 1) / kRedCols));
  k_colreduce<<<grid, kRedThreads, 0, st>>>(op, n, k, A, lda, B, ldb, out); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

int coherit_pcg_state_update(int64_t n, int32_t k, float* X, int64_t ldx, float* R, int64_t ldr,
                             const float* P, int64_t ldp, const float* AP, int64_t ldap,
                             const double* rs, const double* denom, const uint8_t* active,
                             int32_t* breakdown, void* stream) {
  CO_CHECK(k >= 1 && k <= 8192, COHERIT_E_SHAPE, "k=%d outside [1, 8192]", k);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_pcg_state<<<elem_grid(n * k), 256, sizeof(float) * k, st>>>(n, k, X, ldx, R, ldr, P, ldp, AP,
                                                                ldap, rs, denom, active, breakdown); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

int coherit_pcg_direction_update(int64_t n, int32_t k, float* P, int64_t ldp, const float* Z,
                                 int64_t ldz, const double* rs_new, const double* rnorm2,
                                 double* rs_old, const double* threshold, uint8_t* active,
                                 double* rnorm_out, void* stream) {
  CO_CHECK(k >= 1 && k <= 4096, COHERIT_E_SHAPE, "k=%d outside [1, 4096]", k);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_pcg_dir<<<elem_grid(n * k), 256, 2 * sizeof(float) * k, st>>>(n, k, P, ldp, Z, ldz, rs_new,
                                                                  rnorm2, rs_old, threshold); note_launch();
  k_pcg_dir_scalars<<<(k + 127) / 128, 128, 0, st>>>(k, rs_new, rnorm2, rs_old, threshold, active,
                                                     rnorm_out); note_launch();
  CO_CUDA(cudaGetLastError());
  return COHERIT_OK;
}

// Runs the one-tile MMA self-test and copies D (128 x 16, row-major) to
// out_host.  Synchronises the stream.  Returns COHERIT_E_TIMEOUT if the
// commit barrier did not complete in time.
int coherit_selftest_mma(int32_t variant, float* out_host, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float* d_out = nullptr;
  int* d_err = nullptr;
  CO_CUDA(cudaMalloc(&d_out, sizeof(float) * 128 * 16));
  CO_CUDA(cudaMalloc(&d_err, sizeof(int)));
  cudaMemsetAsync(d_out, 0xFF, sizeof(float) * 128 * 16, st);
  cudaMemsetAsync(d_err, 0, sizeof(int), st);
  k_probe_mma<<<1, 128, 0, st>>>(variant, d_out, d_err); note_launch();
  cudaError_t e = cudaGetLastError();
  int err = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out_host, d_out, sizeof(float) * 128 * 16, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_out);
  cudaFree(d_err);
  if (e != cudaSuccess) return cuda_status(e, "MMA self-test");
  if (err != 0) {
    set_error("MMA self-test: commit barrier wait timed out");
    return COHERIT_E_TIMEOUT;
  }
  return COHERIT_OK;
}

}  // extern "C"
