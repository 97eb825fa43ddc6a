"""Minimal PLINK 1 BED source (variant-major, memory-mapped).

BED bytes hold 4 samples per byte, sample i at bits 2*(i%4); the 2-bit BED
codes map to A1 allele counts 0->2, 1->missing, 2->1, 3->0
(geno_stream.py:709-745 of the reference).  ``.fam`` and ``.bim`` give the
sample and variant counts.
"""
from __future__ import annotations

import os

import numpy as np

_MAGIC = bytes([0x6C, 0x1B, 0x01])
MISSING_VAL = -127


def _count_lines(path: str) -> int:
    with open(path, "rb") as f:
        return sum(1 for line in f if line.strip())


class BedSource:
    def __init__(self, bed_prefix: str):
        prefix = bed_prefix[:-4] if bed_prefix.endswith(".bed") else bed_prefix
        self._bed_prefix = prefix
        self.n = _count_lines(prefix + ".fam")
        self.m = _count_lines(prefix + ".bim")
        with open(prefix + ".fam") as f:
            self.sample_ids = tuple(line.split()[1] for line in f if line.strip())
        path = prefix + ".bed"
        self._bytes_per_snp = (self.n + 3) // 4
        size = os.path.getsize(path)
        if size != 3 + self._bytes_per_snp * self.m:
            raise ValueError(f"{path}: size {size} does not match n={self.n}, m={self.m}")
        self._mm = np.memmap(path, dtype=np.uint8, mode="r")
        if bytes(self._mm[:3]) != _MAGIC:
            raise ValueError(f"{path}: not a SNP-major PLINK BED file")
        self.missing_val = MISSING_VAL
        lut = np.asarray([2, MISSING_VAL, 1, 0], dtype=np.int8)
        self._lut = lut

    def raw_bytes(self) -> np.ndarray:
        """The whole .bed file (header + SNP-major records), memory-mapped."""
        return self._mm

    def read_block_variant_major(self, start: int, count: int) -> np.ndarray:
        bps = self._bytes_per_snp
        raw = np.asarray(self._mm[3 + start * bps: 3 + (start + count) * bps]).reshape(count, bps)
        codes = np.stack([(raw >> s) & 3 for s in (0, 2, 4, 6)], axis=2).reshape(count, -1)
        return self._lut[codes[:, : self.n]]

    def close(self) -> None:
        self._mm = None


def write_bed(prefix: str, genotypes: np.ndarray) -> None:
    """Write (n, m) allele counts (0/1/2, negative = missing) as a BED triplet."""
    g = np.asarray(genotypes)
    n, m = g.shape
    inv = np.full(g.shape, 1, dtype=np.uint8)  # missing
    inv[g == 2] = 0
    inv[g == 1] = 2
    inv[g == 0] = 3
    bps = (n + 3) // 4
    pad = np.full((m, 4 * bps), 0, dtype=np.uint8)
    pad[:, :n] = inv.T
    q = pad.reshape(m, bps, 4)
    body = (q[:, :, 0] | (q[:, :, 1] << 2) | (q[:, :, 2] << 4) | (q[:, :, 3] << 6)).astype(np.uint8)
    with open(prefix + ".bed", "wb") as f:
        f.write(_MAGIC)
        f.write(body.tobytes())
    with open(prefix + ".fam", "w") as f:
        for i in range(n):
            f.write(f"F{i} I{i} 0 0 0 -9\n")
    with open(prefix + ".bim", "w") as f:
        for j in range(m):
            f.write(f"1 rs{j} 0 {j + 1} A C\n")
