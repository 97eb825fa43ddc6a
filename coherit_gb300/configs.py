"""Workload definitions of the benchmark configurations (synthetic data).

c1  single-GRM REML, n=2000 x m=10000, seed 0, h2=0.5 from 1000 causal SNPs,
    X = [1, 2 N(0,1)], 30 Rademacher probes, 30-step Lanczos, PCG tol 1e-6.
c2  single-GRM REML at scale, n=50000 x m=500000, h2=0.3 from 5000 causal,
    10 N(0,1) covariates (+ intercept), 64 Rademacher probes (a 65-column
    block with the phenotype), BF16 genotype tiles, FP32 PCG, FP64
    Lanczos/AI.
c3  8-component REML, n=100000 x m=1000000, genotypes with block LD (AR(1)
    latent haplotypes in blocks of 200 SNPs, rho ~ U(0, 0.9)), components =
    4 MAF bins x 2 LD-score halves (arbitrary variant groups), 128 probes,
    per-component h2 ~ Dirichlet(1) x 0.4.
c3s single-GRM REML at the c3 size (n=100000 x m=1000000, MAF/HWE
    generator), otherwise the c2 form: h2=0.3, 64 probes, 10 covariates.
    This is the size the 10x fits/hr target is quoted at; an 8-component
    fit at this size takes minutes, a single-GRM batch seconds.
c4  serving stream: 512 fits over one resident n=200000 x m=600000 matrix,
    h2 ~ U(0.05, 0.8), sample subsets ~ LogUniform(1e4, 2e5), 1-20 covariates,
    Poisson arrivals.
c5  SMILE block-weighted GRM, n=100000 x m=300000, 600 blocks of 500 SNPs,
    64-RHS batched V^-1 solves.
Genotypes come from the counter-based MAF/HWE generator (coherit_gb300.synth).
"""
from __future__ import annotations

import dataclasses


@dataclasses.dataclass(frozen=True)
class REMLWorkload:
    name: str
    n: int
    m: int
    h2: float
    n_causal: int
    n_covar: int
    slq_samples: int
    slq_m: int
    pcg_tol: float
    seed: int = 0
    components: tuple | None = None
    precond_rank: int = 0
    minq_iter: int = 20
    # "maf_ld": genotypes with block LD and components from the 4 MAF bins x
    # 2 LD-score halves partition (built by synth.ld_partition_device).
    partition: str | None = None
    ld_block: int = 200
    h2_dirichlet_total: float = 0.0


C1 = REMLWorkload("c1_n2000_m10000", n=2000, m=10000, h2=0.5, n_causal=1000, n_covar=2,
                  slq_samples=30, slq_m=30, pcg_tol=1e-6, seed=0, precond_rank=0)
C2 = REMLWorkload("c2_n50000_m500000", n=50000, m=500000, h2=0.3, n_causal=5000, n_covar=10,
                  slq_samples=64, slq_m=30, pcg_tol=1e-5, seed=1, precond_rank=256)
C3 = REMLWorkload("c3_n100000_m1000000_G8_mafld", n=100000, m=1000000, h2=0.4,
                  n_causal=10000, n_covar=10, slq_samples=128, slq_m=30, pcg_tol=1e-5, seed=2,
                  precond_rank=256, partition="maf_ld", ld_block=200, h2_dirichlet_total=0.4)
C3S = REMLWorkload("c3s_n100000_m1000000_G1", n=100000, m=1000000, h2=0.3, n_causal=10000,
                   n_covar=10, slq_samples=64, slq_m=30, pcg_tol=1e-5, seed=3, precond_rank=256)

# c4's requests are drawn per request by the stream (h2, subset, covariates);
# h2 / n_causal / n_covar here are the generator's defaults for full fits.
C4 = REMLWorkload("c4_n200000_m600000", n=200000, m=600000, h2=0.3, n_causal=5000, n_covar=10,
                  slq_samples=64, slq_m=30, pcg_tol=1e-5, seed=4, precond_rank=256)
C4_SUBSET_MIN = 10000

WORKLOADS = {"c1": C1, "c2": C2, "c3": C3, "c3s": C3S, "c4": C4}
