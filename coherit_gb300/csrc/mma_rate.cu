// mma_rate.cu -- measured issue rate of the operator's tensor-core
// instructions (tcgen05.mma, M = 128, A in tensor memory, B in shared
// memory): the ceiling that bounds narrow operator launches.
//
// One CTA per SM (the dynamic shared-memory request pins one CTA per SM).
// One or two threads of the CTA (lane 0 of warps 0 and 1, which sit on
// different SM sub-partitions) each issue `iters` back-to-back MMAs of width
// N into an accumulator of their own, on zero operands, then one commit and
// one bounded wait.  Cycles per instruction of one issuer come from clock64
// around its issue loop and commit wait in CTA 0; the aggregate rate from
// CUDA events around the launch.  Two issuers at the rate of one would mean
// the tensor pipe, not the issuing thread, sets the pace.
#include "coherit_internal.cuh"
#include "tc_ptx.cuh"

namespace coherit {
namespace {

constexpr int kRateSmem = 150 * 1024;  // > half the SM's shared memory: one CTA per SM
constexpr uint32_t kRateACol = 480;    // A operand: tensor-memory columns [480, 512)
constexpr uint32_t kRateAcc1 = 224;    // second issuer's accumulator column

__global__ void __launch_bounds__(128, 1) k_mma_rate(int kind, int N, int iters, int issuers,
                                                      int* err, unsigned long long* cyc) {
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ uint64_t done[2];
  __shared__ uint32_t tslot;
  // B operand: N rows x 32 bytes of K in 16-byte core matrices (LBO 128,
  // SBO 256); zero-filled.
  for (int i = threadIdx.x; i < 8192 / 4; i += 128) reinterpret_cast<uint32_t*>(sm)[i] = 0u;
  if (threadIdx.x == 0) {
    ptx::mbar_init(&done[0], 1);
    ptx::mbar_init(&done[1], 1);
    ptx::fence_barrier_init();
  }
  ptx::fence_proxy_async_smem();
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (warp == 0) ptx::tmem_alloc(&tslot, 512);
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = tslot;
  {
    // Zero A: every warp its own 32 lanes of columns [480, 512).
    uint32_t z[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) z[i] = 0u;
    ptx::tmem_st32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + kRateACol, z);
    ptx::tmem_wait_st();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  volatile int no_abort = 0;
  if (warp < issuers && lane == 0) {
    const uint64_t bdesc = ptx::smem_desc(ptx::smem_addr(sm), 128u, 256u);
    const uint32_t idesc = kind == 1 ? ptx::idesc_e4m3_f32(128, N) : ptx::idesc_bf16_f32(128, N);
    const uint32_t acc = tmem + (warp == 0 ? 0u : kRateAcc1);
    const unsigned long long t0 = clock64();
    for (int i = 0; i < iters; ++i) {
      const uint32_t a = i == 0 ? 0u : 1u;
      if (kind == 1)
        ptx::mma_ts_f8(acc, tmem + kRateACol, bdesc, idesc, a);
      else
        ptx::mma_ts(acc, tmem + kRateACol, bdesc, idesc, a);
    }
    ptx::mma_commit(&done[warp]);
    ptx::mbar_wait(&done[warp], 0, err, 41, &no_abort);
    const unsigned long long t1 = clock64();
    if (blockIdx.x == 0 && warp == 0) *cyc = t1 - t0;
  }
  __syncwarp();
  for (int i = 0; i < issuers; ++i) ptx::mbar_wait(&done[i], 0, err, 42, &no_abort);
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 512);
  }
}

}  // namespace
}  // namespace coherit

using namespace coherit;

extern "C" int coherit_mma_rate(int32_t kind, int32_t n_cols, int32_t issuers, int32_t iters,
                                double* cycles, double* ms, void* stream) {
  CO_CHECK(kind == 0 || kind == 1, COHERIT_E_SHAPE, "kind must be 0 (BF16) or 1 (E4M3)");
  CO_CHECK(issuers == 1 || issuers == 2, COHERIT_E_SHAPE, "issuers must be 1 or 2");
  CO_CHECK(n_cols >= 16 && n_cols % 16 == 0 &&
               n_cols <= static_cast<int>(issuers == 1 ? 256u : kRateAcc1),
           COHERIT_E_SHAPE, "n_cols must be a multiple of 16 in [16, %d]",
           issuers == 1 ? 256 : static_cast<int>(kRateAcc1));
  CO_CHECK(iters >= 1 && iters <= (1 << 20), COHERIT_E_SHAPE, "iters must lie in [1, 2^20]");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  CO_CUDA(cudaGetDevice(&dev));
  CO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int* d_err = nullptr;
  unsigned long long* d_cyc = nullptr;
  CO_CUDA(cudaMalloc(&d_err, sizeof(int)));
  cudaError_t e = cudaMalloc(&d_cyc, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(int), st);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mma_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, kRateSmem);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    k_mma_rate<<<sms, 128, kRateSmem, st>>>(kind, n_cols, 64, issuers, d_err, d_cyc);  // warm
    note_launch();
    e = cudaEventRecord(e0, st);
  }
  if (e == cudaSuccess) {
    k_mma_rate<<<sms, 128, kRateSmem, st>>>(kind, n_cols, iters, issuers, d_err, d_cyc);
    note_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float t = 0.f;
  int herr = 0;
  unsigned long long hc = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&hc, d_cyc, sizeof(hc), cudaMemcpyDeviceToHost);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d_err);
  cudaFree(d_cyc);
  if (e != cudaSuccess) return cuda_status(e, "mma rate");
  CO_CHECK(herr == 0, COHERIT_E_TIMEOUT, "mma rate kernel wait ran out (code %d)", herr);
  if (cycles) *cycles = static_cast<double>(hc) / iters;
  if (ms) *ms = t;
  return COHERIT_OK;
}
