// op_noalloc.cu -- genotype operator whose workspace is a fixed static
// device array, so a call allocates no device memory.
//
// coherit_geno_kv places its workspace (BF16 split tiles of V and S, column
// sums, rank-one terms, missing-genotype corrections) in a per-handle buffer
// that grows with cudaMalloc on the first call of a wider shape, and growing
// it frees the old buffer after a device-wide synchronisation.  This variant
// runs the same launches with the workspace in `g_scratch` below instead.
//
// Setup: the first call on each device, with that device current, resolves
// the array's address with cudaGetSymbolAddress and caches it; later calls
// only read the cache.  Make that first call before any stream capture
// begins.  Under lazy module loading (the CUDA default) that first call loads
// the module holding the array and commits its 64 MiB; with eager loading
// (CUDA_MODULE_LOADING=EAGER) every context that loads this library commits
// 64 MiB on each device it uses, whether or not this entry point is called.
//
// Limits: single request, tensor-core precisions; the workspace of one
// launch (about 2*nsplit*kp*(n_pad + m_pad) bytes, plus 8*kp*m_pad with
// missing genotypes, plus the split-K partials) must fit kScratchBytes, else
// COHERIT_E_SHAPE.
//
// What must start at zero: the FP64 rank-one accumulators and the FP16X2
// column maxima, cleared by the launch sequence on every call; every other
// region is written before it is read.  Calls on one device share the array:
// calls issued on one stream (or otherwise ordered, e.g. with events) are
// safe, calls in flight at the same time on different streams race on it.
#include <mutex>

#include "coherit_internal.cuh"

namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int scratch_for_device(int device, void** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (g_scratch_ptr[device] == nullptr) {
    void* p = nullptr;
    CO_CUDA(cudaGetSymbolAddress(&p, g_scratch));
    g_scratch_ptr[device] = p;
  }
  *out = g_scratch_ptr[device];
  return COHERIT_OK;
}

}  // namespace

using namespace coherit;

extern "C" int coherit_geno_kv_noalloc(coherit_geno_t* h, int32_t slot, int32_t mode,
                                       int32_t precision, const float* V, int64_t ldv, int32_t k,
                                       const float* comp_scale, int32_t use_theta_e,
                                       float theta_e, const float* snp_weight, float* out,
                                       int64_t ldo, void* stream) {
  CO_CHECK(h != nullptr, COHERIT_E_CLOSED, "genotype handle is closed");
  CO_CHECK(k >= 1, COHERIT_E_SHAPE, "right-hand side must have at least one column");
  CO_CHECK(slot >= 0 && slot < static_cast<int32_t>(h->slots.size()) && h->slots[slot].used,
           COHERIT_E_INDEX, "stats slot %d is not initialised", slot);
  CO_CHECK(mode == COHERIT_MODE_SUM || mode == COHERIT_MODE_STACKED, COHERIT_E_SHAPE,
           "unknown operator mode %d", mode);
  CO_CHECK(ldv >= k && ldo >= k, COHERIT_E_SHAPE, "row strides must be >= k");
  CO_CHECK(V != nullptr && out != nullptr, COHERIT_E_SHAPE, "V and out are required");
  CO_CHECK(h->device >= 0 && h->device < kMaxDevices, COHERIT_E_UNSUPPORTED,
           "device ordinal %d out of range", h->device);
  int cur = -1;
  CO_CUDA(cudaGetDevice(&cur));
  CO_CHECK(cur == h->device, COHERIT_E_SHAPE,
           "device %d must be current for a handle on device %d", h->device, h->device);
  void* scratch = nullptr;
  int rc = scratch_for_device(h->device, &scratch);
  if (rc != COHERIT_OK) return rc;

  OpDesc d;
  d.n_groups = 1;
  d.col_start = {0, k};
  d.slot_of_group = {slot};
  d.comp_scale.assign(h->G, 1.f);
  if (comp_scale != nullptr)
    for (int g = 0; g < h->G; ++g) d.comp_scale[g] = comp_scale[g];
  d.k = k;
  d.mode = mode;
  d.precision = precision;
  if (use_theta_e && mode == COHERIT_MODE_SUM) d.theta_e = {theta_e};
  d.snp_weight = snp_weight;
  d.V = V;
  d.ldv = ldv;
  d.out = out;
  d.ldo = ldo;
  return run_operator_in_scratch(h, d, scratch, kScratchBytes, static_cast<cudaStream_t>(stream));
}
