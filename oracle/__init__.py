"""CPU oracle for the COHERIT/GPU_REML matrix-free REML hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in ``coherit_gb300`` imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline / reference arm use it, and only as the checker or the timed
CPU restatement, never as the measured GPU path.

The reference (a JAX + numba package) cannot run in this environment (jax,
jaxlib, numba and bed_reader are absent), so every function here restates
the reference's published algorithm in numpy and cites the reference file
and lines it follows:

* ``geno``    -- packed 2-bit format, call geometry, FP32 per-SNP statistics,
                 the genotype operator in FP64 (and the FP32 streamed form of
                 kv_impl.py used as the CPU baseline).
* ``pcg``     -- block PCG (pcg.py).
* ``precond`` -- projected-core preconditioner (precond.py).
* ``slq``     -- SLQ log-determinant value and exact gradient (slq.py) and
                 the affine single-GRM cache (reml.py).
* ``reml``    -- REML evaluation, AI/NNLS step and the strict fit loop
                 (reml.py).
* ``synth``   -- the synthetic genotype/phenotype generators of the
                 benchmark configurations (counter-based hash shared with the
                 CUDA generator).

Parity pinning: the reference ships no golden vectors.  The oracle is pinned
against the known-answer checks of the reference's own tests, restated in
``tests/test_oracle_pins.py`` (diagonal and dense PCG solves, zero and
extreme right-hand sides, full-depth SLQ equal to the dense probe quadratic
form, SLQ gradients equal to finite differences, affine-SLQ score equal to
the finite difference of the REML objective), and the operator against a
dense FP64 GRM (the validation the reference's docs prescribe).  Probe
values of ``jax.random`` are not reproduced: both sides receive the same
probe matrices instead ("parity unpinned" for the PRNG stream only).
"""
