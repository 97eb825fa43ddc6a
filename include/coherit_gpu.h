/*
 * coherit_gpu.h -- C ABI of the GB300 (sm_103a) genotype-operator library.
 *
 * The library owns 2-bit packed genotypes resident in HBM and applies the
 * standardised genomic-relationship operator of COHERIT/GPU_REML to blocks of
 * right-hand sides:
 *
 *     K V = sum_b Z_b (Z_b^T V) / m_eff          (kv_impl.py:9-12)
 *
 * where Z_b is the mean-imputed, centred, 1/sd-scaled genotype slice of call
 * block b (kv_impl.py:69-91).  Every entry point takes plain pointers and
 * sizes; device pointers are CUDA device addresses on the handle's device and
 * `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * All device work is enqueued on `stream`; no entry point synchronises the
 * stream unless its comment says so.
 *
 * Every function returns a status code (COHERIT_OK on success).  The Python
 * layer maps them onto the exception types of the reference:
 *   COHERIT_E_SHAPE          -> ValueError      (geno_stream.py:1188-1252, kv_impl.py:538-571)
 *   COHERIT_E_INDEX          -> IndexError      (geno_stream.py:2687-2690)
 *   COHERIT_E_NONFINITE      -> FloatingPointError (pcg.py:117-119)
 *   COHERIT_E_NOT_CONVERGED  -> FloatingPointError (reml.py:770-776)
 *   COHERIT_E_CLOSED         -> RuntimeError    (geno_stream.py:2610-2614)
 *   COHERIT_E_OOM, _CUDA, _TIMEOUT, _UNSUPPORTED -> RuntimeError / MemoryError
 * coherit_last_error() returns a thread-local message for the last failure.
 */
#ifndef COHERIT_GPU_H
#define COHERIT_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COHERIT_OK 0
#define COHERIT_E_SHAPE 1
#define COHERIT_E_NONFINITE 2
#define COHERIT_E_NOT_CONVERGED 3
#define COHERIT_E_OOM 4
#define COHERIT_E_TIMEOUT 5
#define COHERIT_E_CLOSED 6
#define COHERIT_E_CUDA 7
#define COHERIT_E_INDEX 8
#define COHERIT_E_UNSUPPORTED 9

/* Arithmetic of one operator application.
 *  FP32    : CUDA-core FP32 decode/centre/two contractions; the "plain FP32"
 *            form of the reference's Precision.HIGHEST matmuls (kv_impl.py:107-113).
 *  BF16X3  : tcgen05 tensor cores, genotypes exact in BF16, right-hand sides
 *            split into three BF16 terms (~FP32 accuracy), FP32 accumulation.
 *  BF16X2 / BF16X1 : fewer split terms (faster, less accurate; for sketches).
 *  FP16X2  : tcgen05 tensor cores, genotypes exact in FP16, right-hand sides
 *            (and the intermediate S) scaled per column by a power of two and
 *            split into two FP16 terms (22 significant bits), FP32
 *            accumulation; two terms instead of three, so one instruction of
 *            N = 256 carries 128 columns. */
#define COHERIT_PREC_FP32 0
#define COHERIT_PREC_BF16X3 1
#define COHERIT_PREC_BF16X2 2
#define COHERIT_PREC_BF16X1 3
#define COHERIT_PREC_FP16X2 4
/*  FP8X5   : tcgen05 kind::f8f6f4 tensor cores, genotypes exact in E4M3,
 *            right-hand sides (and S) scaled per column by a power of two and
 *            split into five E4M3 terms (term t holds the previous residual
 *            times 16; ~20 significant bits), FP32 accumulation; K = 32 per
 *            instruction, half the instructions of the 16-bit forms, for
 *            blocks of <= 48 columns. */
#define COHERIT_PREC_FP8X5 5
/*  AUTO    : per launch, FP8X5 for blocks of <= 48 columns (half the MMA
 *            instructions where their count bounds the time) and BF16X3 for
 *            wider blocks; both hold the 1e-5 operator bound. */
#define COHERIT_PREC_AUTO 6

/* Operator output forms. */
#define COHERIT_MODE_SUM 0      /* out = sum_g scale_g K_g V (+ theta_e V)         */
#define COHERIT_MODE_STACKED 1  /* out[g] = scale_g K_g V, shape (G, n, k)          */

typedef struct coherit_geno coherit_geno_t;

const char* coherit_last_error(void);
int coherit_version(void);
/* Number of kernels the library has launched in this process (no counterpart
 * in the reference; lets callers count device work inside a timed region). */
int64_t coherit_launch_count(void);
/* Number of devices and whether device `dev` is a tcgen05-capable part. */
int coherit_device_info(int dev, int* sm_major, int* sm_minor, int* n_sm, int64_t* hbm_bytes);

/* ---------------------------------------------------------------- genotypes */

/* Build the resident genotype matrix from the reference's packed cache.
 * Replaces GenoBlockStreamer's tmpfile/ring cache (geno_stream.py:1323-1331,
 * :2358-2396) and its per-call H2D streaming (kv_impl.py:300-320).
 *   packed            : concatenation over calls c of row-major (n, ceil(w_c/4))
 *                       uint8 blocks; SNP 4j+s of a row sits at bits 2s..2s+1 of
 *                       byte j; codes 0/1/2 = allele count, 3 = missing
 *                       (kv_impl.py:58-66, geno_stream.py:1263).  Host memory
 *                       unless packed_on_device != 0.
 *   call_widths       : n_calls true widths (geno_stream.py:1303)
 *   call_component_ids: n_calls component ids (NULL = all component 0);
 *                       calls of one component must be contiguous
 *                       (geno_stream.py:469-505).                              */
int coherit_geno_create_packed(const uint8_t* packed, int64_t n, int32_t n_calls,
                               const int32_t* call_widths, const int32_t* call_component_ids,
                               int32_t n_components, int packed_on_device, int device,
                               void* stream, coherit_geno_t** out);

/* Build the resident matrix directly from a PLINK 1 SNP-major .bed file held
 * in host memory (`bed`, `bed_bytes` bytes including the 3-byte header; n_full
 * samples, m SNP records), transcoding BED codes 0,1,2,3 to allele counts
 * 2, missing, 1, 0 on the device in chunks of whole SNP records.  keep: host
 * list of n_keep source sample indices to retain (NULL = all).  Components as
 * in coherit_geno_create_synthetic (contiguous SNP ranges).  Replaces the
 * host transcode of the reference's cache build (geno_stream.py:709-745,
 * :1594-1846).  Synchronises `stream`.                                       */
int coherit_geno_create_bed(const uint8_t* bed, int64_t bed_bytes, int64_t n_full, int64_t m,
                            const int32_t* keep, int64_t n_keep, const int32_t* component_sizes,
                            int32_t n_components, int device, void* stream,
                            coherit_geno_t** out);

/* Benchmark genotypes with linkage disequilibrium, generated on the device
 * (no counterpart in the reference, which reads real genotype files; this
 * builds the synthetic 8-component workload: SNPs in blocks of `block`, two
 * latent AR(1) haplotype chains per sample and block,
 * x_p = rho_b x_{p-1} + s_b e_p in FP32, allele = [x_p < thresholds[j]],
 * e from the 4096-entry standard-normal quantile table `quantiles` indexed
 * by a counter-based hash of (seed, SNP, sample, haplotype)).
 *
 * coherit_ldblock_records writes SNP-major PLINK BED records (m records of
 * ceil(n_rows/4) bytes) for samples 0..n_rows-1 into the device buffer
 * `out`; the tables are device arrays (thresholds: m, rho and sfac:
 * ceil(m/block), quantiles: 4096).  Used for LD scores on a sample prefix.
 *
 * coherit_geno_create_ldblock builds the resident matrix of n samples from
 * the same generator with host tables; cache_to_source (host, m entries,
 * NULL = identity) places source SNP cache_to_source[c] at cache position c,
 * so arbitrary variant groups become contiguous components of
 * component_sizes.  Synchronises `stream`.                                    */
int coherit_ldblock_records(int64_t n_rows, int64_t m, int32_t block, uint64_t seed,
                            const float* thresholds, const float* rho, const float* sfac,
                            const float* quantiles, uint8_t* out, void* stream);
int coherit_geno_create_ldblock(int64_t n, int64_t m, int32_t block, uint64_t seed,
                                const float* thresholds, const float* rho, const float* sfac,
                                const float* quantiles, const int64_t* cache_to_source,
                                const int32_t* component_sizes, int32_t n_components, int device,
                                void* stream, coherit_geno_t** out);

/* Build a synthetic resident matrix (no host copy): per-SNP MAF ~ U(0.05, 0.5)
 * and genotypes ~ Binomial(2, MAF) drawn from a counter-based hash of
 * (seed, snp, sample); `missing_q24` = missing rate * 2^24 (0 = none).  The
 * same generator is restated in the oracle so both see identical genotypes.
 * component_sizes: n_components SNP counts (NULL = one component of m).      */
int coherit_geno_create_synthetic(int64_t n, int64_t m, const int32_t* component_sizes,
                                  int32_t n_components, uint64_t seed, uint32_t missing_q24,
                                  int device, void* stream, coherit_geno_t** out);

int coherit_geno_destroy(coherit_geno_t* h);

/* Shapes: n samples, m SNPs, padded extents of the HBM layout, components,
 * number of missing genotype entries, bytes held on the device.             */
int coherit_geno_info(const coherit_geno_t* h, int64_t* n, int64_t* m, int64_t* n_pad,
                      int64_t* m_pad, int32_t* n_components, int64_t* n_missing,
                      int64_t* device_bytes);

/* Copy back the reference-layout packed bytes of call-sized column range
 * [snp_start, snp_start+width) as a row-major (n, ceil(width/4)) host block
 * (the bytes GenoBlockStreamer._pop_cached returns, geno_stream.py:2605-2617). */
int coherit_geno_read_packed(coherit_geno_t* h, int64_t snp_start, int32_t width,
                             uint8_t* out_host, void* stream);

/* Standardised genotype columns of stats slot `slot`: out[i*ldo + c] =
 * (g_ic - mean) * inv_sd of cache SNP snp_idx[c] (device int64 array of
 * `count` indices) for every sample i, 0 where the genotype is missing,
 * evaluated in FP32 in the reference's order.  out: device, n x ldo.
 * Replaces GenoBlockStreamer.extract_standardized_columns
 * (geno_stream.py:2748-2760, :2472-2502), here on the device.  An index
 * outside [0, m) yields a NaN column.                                        */
int coherit_geno_extract_columns(coherit_geno_t* h, int32_t slot, const int64_t* snp_idx,
                                 int32_t count, float* out, int64_t ldo, void* stream);

/* ------------------------------------------------------------ standardisation */

/* Compute per-SNP statistics of stats slot `slot` over the samples selected by
 * `sample_mask` (n host bytes, nonzero = keep; NULL = all samples), following
 * the reference's FP32 formulas (geno_stream.py:1780-1792):
 *     mean = s1/max(cnt,1); var = max(s2/max(cnt,1) - mean^2, 0);
 *     inv_sd = 1/sqrt(max(var,1e-6)) if cnt>0 and var>0 else 0.
 * Slot 0 is the full-sample slot used by default.  Outputs (host, length m,
 * cache order; any may be NULL): mean, inv_sd, count of observed genotypes.
 * Synchronises `stream`.                                                    */
int coherit_geno_compute_stats(coherit_geno_t* h, int32_t slot, const uint8_t* sample_mask,
                               float* mean_out, float* inv_sd_out, int32_t* count_out,
                               void* stream);

/* Install externally supplied standardisation (standardization_override,
 * geno_stream.py:1283-1292) into slot `slot`.  mean/inv_sd: host, length m. */
int coherit_geno_set_stats(coherit_geno_t* h, int32_t slot, const uint8_t* sample_mask,
                           const float* mean, const float* inv_sd, void* stream);

/* Free a stats slot (slot > 0). */
int coherit_geno_release_stats(coherit_geno_t* h, int32_t slot);

/* Per-component effective SNP counts m_eff (#inv_sd>0) and mean-diagonal atoms
 * tr(K_g)/n of slot `slot` (geno_stream.py:1409-1444); host arrays of length
 * n_components; the totals over all components go to *eff_total / *atom_total.
 */
int coherit_geno_stats_summary(const coherit_geno_t* h, int32_t slot, double* comp_eff,
                               double* comp_atom, double* eff_total, double* atom_total);

/* Exact sample-wise diagonal of the whole-matrix GRM, diag(K)_i =
 * sum_j z_ij^2 / m_eff in FP64 (geno_stream.py:2780-2821).  out: device, n.   */
int coherit_geno_exact_diag(coherit_geno_t* h, int32_t slot, float* out, void* stream);

/* ------------------------------------------------------------------ operator */

/* Reserve the operator workspace for right-hand-side blocks of up to k_max
 * columns so later calls allocate nothing (needed before stream capture).   */
int coherit_geno_reserve(coherit_geno_t* h, int32_t k_max, int32_t precision);

/* Genotype operator on V (device, n x k, row stride ldv floats).
 * MODE_SUM:     out[i,c] = sum_g comp_scale[g] (Z_g Z_g^T V)[i,c] + theta_e V[i,c]
 * MODE_STACKED: out[g*n*ldo + i*ldo + c] = comp_scale[g] (Z_g Z_g^T V)[i,c]
 * comp_scale (host, n_components): per-component multiplier applied to
 * Z_g Z_g^T, e.g. 1/m_eff,g for kv(normalize=True) (kv_impl.py:320-324),
 * theta_g/m_eff,g for the weighted H.V (kv_impl.py:1116-1131).
 * snp_weight: optional device array (m, cache order) of per-SNP kernel weights
 * (kv_impl.py:139-160); NULL = none.
 * Replaces kv_impl_streamed (kv_impl.py:268-326), kv_impl_partitioned_weighted
 * (:1089-1135), kv_impl_partitioned_stacked (:1138-1187),
 * kv_impl_snp_weighted_streamed (:329-379).                                 */
/* Launch-configuration autotuner (no counterpart in the reference, whose
 * jitted kernels have no tunable launch shape).  Times the operator at width
 * k (one launch, <= 80 columns at BF16X3, 48 at FP8X5, 128 at FP16X2) and
 * `precision` (AUTO resolves by width) on this handle's genotypes and stats
 * slot 0 under each candidate configuration -- two- or four-block pipeline
 * stages, tensor-memory A-ring depth, shared-memory B-ring depth, and the
 * grid size (2, 4 or 8 x SMs) the split-K plan fills, one or two row tiles
 * per CTA (two MMA-issuing threads on one B supply), and clusters of 2 CTAs
 * that share each B tile (one multicast copy from L2 instead of one per
 * CTA) -- `reps` timed applications each (CUDA events on `stream`); the
 * fastest three and the fixed policy are timed again with 3 x `reps`, and
 * the fastest is kept for every later launch of that width and precision
 * on the handle.  Allocates and frees two n x k buffers; synchronises
 * `stream`.  Genotype-ring depth is a candidate too (full, or two stages per
 * decoder set where that frees shared memory for another B slot).
 * choice (8 ints, may be NULL): four-block stages (0/1), A-ring slots,
 * B-ring slots, grid multiple, candidates tried, CTAs per cluster,
 * genotype-ring stages, row tiles per CTA;
 * best_ms / default_ms: per-application times of the kept and of the
 * fixed-policy configuration.                                             */
int coherit_geno_autotune(coherit_geno_t* h, int32_t k, int32_t precision, int32_t reps,
                          int32_t* choice, float* best_ms, float* default_ms, void* stream);

/* Pin the launch configuration of width k (rounded up to 16) and
 * `precision` (AUTO resolves by width) on this handle, in place of the fixed
 * policy or a tuned choice (no counterpart in the reference): cfg (8 ints,
 * the layout of coherit_geno_autotune's choice) = four-block stages (0/1),
 * A-ring slots, B-ring slots (0 = largest that fits; depths are clamped to
 * what fits), grid multiple (2, 4 or 8), unused, CTAs per cluster (1 or 2),
 * genotype-ring stages (0 = full; else a multiple of the decoder sets, 2
 * for four-block and 3 for two-block stages), row tiles per CTA (1 or 2;
 * 2 falls back to 1 where both accumulators and rings do not fit; not with
 * clusters).  cfg NULL returns the width to the fixed policy.              */
int coherit_geno_set_launch(coherit_geno_t* h, int32_t k, int32_t precision, const int32_t* cfg);

/* Tensor-core instruction-rate probe (no counterpart in the reference: it
 * measures the ceiling of this library's operator, not a reference step).
 * One CTA per SM; `issuers` (1 or 2) threads per CTA, on different SM
 * sub-partitions, each issue `iters` back-to-back tcgen05.mma of M = 128,
 * N = n_cols (multiple of 16; <= 256 with one issuer, <= 224 with two),
 * A in tensor memory, B in shared memory, kind 0 = BF16 (K = 16) or
 * 1 = E4M3 (K = 32), on zero operands.  cycles: SM cycles per instruction
 * of one issuer of CTA 0; ms: device time of the whole launch (CUDA events
 * on `stream`).  Allocates and frees 12 bytes; synchronises `stream`.       */
int coherit_mma_rate(int32_t kind, int32_t n_cols, int32_t issuers, int32_t iters,
                     double* cycles, double* ms, void* stream);

int coherit_geno_kv(coherit_geno_t* h, int32_t slot, int32_t mode, int32_t precision,
                    const float* V, int64_t ldv, int32_t k, const float* comp_scale,
                    int32_t use_theta_e, float theta_e, const float* snp_weight,
                    float* out, int64_t ldo, void* stream);

/* coherit_geno_kv with the same arguments and results, but the workspace is a
 * fixed 64 MiB static device array instead of the handle's growable buffer,
 * so the call allocates no device memory (no counterpart in the reference).
 * For callers that cannot allocate or free during a solve: the per-handle
 * buffer grows with cudaMalloc on the first wider call, and growing it runs
 * cudaFree after a device-wide synchronisation, which stalls every other
 * stream of the process.  Several solvers sharing a device must order their
 * calls (one stream, or events between streams): they share the array.
 *   - tensor-core precisions only (COHERIT_PREC_FP32 -> COHERIT_E_UNSUPPORTED);
 *   - the workspace of one launch, about 2*nsplit*kp*(n_pad + m_pad) bytes
 *     (+ 8*kp*m_pad with missing genotypes, + the split-K partials; kp =
 *     columns per launch rounded up to 16), must fit 64 MiB, else
 *     COHERIT_E_SHAPE;
 *   - the handle's device must be current; the first call on a device
 *     resolves the array's address (cudaGetSymbolAddress), so make it before
 *     any stream capture; with lazy module loading (the default) that call
 *     commits the 64 MiB, with CUDA_MODULE_LOADING=EAGER every context that
 *     loads the library commits it on each device it uses;
 *   - calls on one device share the array: calls in flight at the same time
 *     on different streams race; calls ordered on one stream are safe.     */
int coherit_geno_kv_noalloc(coherit_geno_t* h, int32_t slot, int32_t mode, int32_t precision,
                            const float* V, int64_t ldv, int32_t k, const float* comp_scale,
                            int32_t use_theta_e, float theta_e, const float* snp_weight,
                            float* out, int64_t ldo, void* stream);

/* Batched operator for independent requests sharing the genotypes: columns
 * [col_start[r], col_start[r+1]) of V belong to request r, which uses stats
 * slot slots[r] (its own sample subset, mean, sd, m_eff), per-component scale
 * comp_scale[r*G + g] and residual weight theta_e[r] (NULL = none).  Rows
 * outside a request's subset are returned as zero; V must be zero there.   */
int coherit_geno_kv_batched(coherit_geno_t* h, int32_t n_requests, const int32_t* col_start,
                            const int32_t* slots, int32_t precision, const float* V,
                            int64_t ldv, int32_t k, const float* comp_scale,
                            const float* theta_e, float* out, int64_t ldo, void* stream);

/* X^T V: out (device, m x k, row stride ldo, cache SNP order) =
 * scale[g(j)] * inv_sd_j * (diff^T V)_j   (kv_impl.py:163-185, :382-439).     */
int coherit_geno_xtv(coherit_geno_t* h, int32_t slot, int32_t precision, const float* V,
                     int64_t ldv, int32_t k, const float* comp_scale, float* out, int64_t ldo,
                     void* stream);

/* Z b: out (device, n x C, row stride ldo) = sum_j diff_ij inv_sd_j b[j,:]
 * for b (device, m x C, row stride ldb, cache order) (kv_impl.py:221-265);
 * replaces zxb_impl_streamed / _same_stream_multi / _multi_streamed
 * (kv_impl.py:524-724), several effect vectors being the C columns.        */
int coherit_geno_zxb(coherit_geno_t* h, int32_t slot, int32_t precision, const float* b,
                     int64_t ldb, int32_t C, float* out, int64_t ldo, void* stream);

/* Device-side error flag: returns COHERIT_E_TIMEOUT if any kernel of this
 * handle gave up on a bounded wait since the last call (and clears it).
 * Synchronises `stream`.                                                    */
int coherit_geno_check(coherit_geno_t* h, void* stream);

/* -------------------------------------------------------- solver primitives */

/* Column reductions over n rows for k columns (device arrays, row strides):
 *   op 0: out[c] = sum_i A[i,c] * B[i,c]     op 1: out[c] = sum_i A[i,c]^2
 * accumulated in FP64; out is device, k doubles.                            */
int coherit_colreduce(int32_t op, int64_t n, int32_t k, const float* A, int64_t lda,
                      const float* B, int64_t ldb, double* out, void* stream);

/* Fused block-PCG state update (pcg.py:31-48): given the column sums
 * denom = sum(P*AP), rs and the active mask, computes
 * alpha = active&valid ? rs/denom : 0, X += P alpha, R -= AP alpha, and sets
 * *breakdown (device int) if an active column had a non-positive or
 * non-finite curvature. rs/denom device doubles, active device uint8.        */
int coherit_pcg_state_update(int64_t n, int32_t k, float* X, int64_t ldx, float* R,
                             int64_t ldr, const float* P, int64_t ldp, const float* AP,
                             int64_t ldap, const double* rs, const double* denom,
                             const uint8_t* active, int32_t* breakdown, void* stream);

/* Fused block-PCG direction update (pcg.py:51-65): given rs_new = sum(R*Z),
 * rnorm^2 = sum(R*R), rs_old and threshold, writes active = rnorm > thr,
 * beta = active ? rs_new/(rs_old>0 ? rs_old : 1) : 0, P = active ? Z + P beta : 0,
 * rs_old <- active ? rs_new : 0, rnorm_out <- sqrt(rnorm^2).                  */
int coherit_pcg_direction_update(int64_t n, int32_t k, float* P, int64_t ldp,
                                 const float* Z, int64_t ldz, const double* rs_new,
                                 const double* rnorm2, double* rs_old, const double* threshold,
                                 uint8_t* active, double* rnorm_out, void* stream);

/* Projected-core preconditioner apply (precond.py:42-84): out = a V + U (G
 * (U^T V)) for the basis U (device, n x r, row stride ldu), the r x r core
 * G (device, row stride ldg) and V (device, n x k), in the library's own
 * kernels (FP32, the slice sums of U^T V in FP64).  M^{-1} V takes
 * G = (dI + C)^{-1} - d^{-1} I and a = 1/d; M^{-1/2} V takes
 * G = Q diag(e^{-1/2}) Q^T - d^{-1/2} I and a = d^{-1/2}.  work: device
 * scratch of coherit_lowrank_workspace_floats(n, r, k) floats.  Replaces
 * _apply_scalar_diag / _apply_invsqrt (precond.py:42-84).                   */
int coherit_lowrank_workspace_floats(int64_t n, int32_t r, int32_t k, int64_t* floats);
int coherit_lowrank_apply(int64_t n, int32_t r, int32_t k, const float* U, int64_t ldu,
                          const float* G, int64_t ldg, float a, const float* V, int64_t ldv,
                          float* out, int64_t ldo, float* work, int64_t work_floats,
                          void* stream);

/* ------------------------------------------- rare-variant sparse operator */

/* Rare-variant ("sparse12") genotype matrix: per-SNP lists of the non-zero
 * genotypes (het = 1, hom-alt = 2, missing = 3, samples ascending) resident
 * in HBM, replacing SparseGenoBlockStreamer's host CSC shards and their
 * per-pass device_put (sparse_stream.py:804-1222).                          */
typedef struct coherit_sparse coherit_sparse_t;

/* Build from a PLINK 1 SNP-major .bed held in host memory (layout and keep
 * list as coherit_geno_create_bed), counting and then filling the entries on
 * the device in chunks of whole SNP records (the single-pass raw-BED build of
 * sparse_stream.py:518-606, :711-801).  Synchronises `stream`.              */
int coherit_sparse_create_bed(const uint8_t* bed, int64_t bed_bytes, int64_t n_full, int64_t m,
                              const int32_t* keep, int64_t n_keep, int device, void* stream,
                              coherit_sparse_t** out);

/* Build a synthetic rare-variant matrix on the device (no host copy): per-SNP
 * MAF ~ U[maf_lo_q24, maf_hi_q24) / 2^24 and genotypes ~ Binomial(2, MAF)
 * from the counter-based hash of coherit_geno_create_synthetic (same key per
 * (seed, snp, sample)), `missing_q24` = missing rate * 2^24.  The generator
 * is restated in the oracle.  Synchronises `stream`.                        */
int coherit_sparse_create_synthetic(int64_t n, int64_t m, uint64_t seed, uint32_t maf_lo_q24,
                                    uint32_t maf_hi_q24, uint32_t missing_q24, int device,
                                    void* stream, coherit_sparse_t** out);

/* Build from host entry lists (any other genotype source): col_off[m+1]
 * offsets, rows[nnz] sample indices < n, vals[nnz] in {1, 2, 3}
 * (the packed het/hom/missing orders of sparse_stream.py:671-708).          */
int coherit_sparse_create_csc(int64_t n, int64_t m, const int64_t* col_off, const int32_t* rows,
                              const int8_t* vals, int device, void* stream,
                              coherit_sparse_t** out);

int coherit_sparse_destroy(coherit_sparse_t* h);

/* Samples, SNPs, stored entries, missing entries, bytes held on the device. */
int coherit_sparse_info(const coherit_sparse_t* h, int64_t* n, int64_t* m, int64_t* nnz,
                        int64_t* n_missing, int64_t* device_bytes);

/* Host copies of the FP32 mean / inverse sd and the het / hom / missing
 * counts (m each, any may be NULL), m_eff (SNPs with inv > 0) and the mean
 * diagonal atom (sparse_stream.py:726-742, geno_stream.py:1409-1420).      */
int coherit_sparse_stats(const coherit_sparse_t* h, float* mean, float* inv, int64_t* n_het,
                         int64_t* n_hom, int64_t* n_miss, double* eff_m, double* mean_diag_atom);

/* Install caller-supplied FP32 mean / inverse sd (host, m each), e.g. the
 * statistics a shard payload carries (sparse_stream.py:1037-1145); m_eff,
 * the mean-diagonal atom and the exact-diagonal base follow them.
 * Synchronises `stream`.                                                    */
int coherit_sparse_set_stats(coherit_sparse_t* h, const float* mean, const float* inv,
                             void* stream);

/* Host copy of the entries: col_off[m+1], rows[nnz], vals[nnz].            */
int coherit_sparse_read_csc(const coherit_sparse_t* h, int64_t* col_off, int32_t* rows,
                            int8_t* vals);

/* out (n x k, ldo) = scale * Z Z^T V + theta_e * V for device V (n x k, ldv)
 * (kv_impl.py:777-905, sparse_stream.py:1344-1388 with scale = theta/m_eff).
 * out must not alias V.  Asynchronous on `stream`.                         */
int coherit_sparse_kv(coherit_sparse_t* h, const float* V, int64_t ldv, int32_t k, double scale,
                      float theta_e, float* out, int64_t ldo, void* stream);

/* out (m x k, ldo) = scale * Z^T V (kv_impl.py:752-827,
 * sparse_stream.py:1390-1421).  Asynchronous on `stream`.                  */
int coherit_sparse_xtv(coherit_sparse_t* h, const float* V, int64_t ldv, int32_t k, double scale,
                       float* out, int64_t ldo, void* stream);

/* Standardised FP32 columns (n x count, ldo) of the SNPs in device array
 * snp_idx; missing genotypes give 0, an index outside [0, m) gives a NaN
 * column (sparse_stream.py:893-961).                                        */
int coherit_sparse_extract_columns(coherit_sparse_t* h, const int64_t* snp_idx, int32_t count,
                                   float* out, int64_t ldo, void* stream);

/* Exact diagonal of Z Z^T / m_eff into device out[n], accumulated in FP64
 * (geno_stream.py:2780-2821).                                               */
int coherit_sparse_exact_diag(coherit_sparse_t* h, float* out, void* stream);

/* One-tile tensor-core self-test (no counterpart in the reference): computes
 * D(128x16) = A(128x16) B(16x16)^T for fixed small integers with A taken from
 * tensor memory (variant 0) or shared memory (variant 1) and copies D to
 * out_host (128*16 floats, row-major).  Synchronises `stream`.              */
int coherit_selftest_mma(int32_t variant, float* out_host, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* COHERIT_GPU_H */
