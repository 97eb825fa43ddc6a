"""SMILE-style block-weighted GRM operators on the resident genotype matrix.

One genetic kernel of the form

    K V = sum_b Z_b W_b Z_b^T V / c                     (smile_block_w.py:1-14)

for contiguous SNP blocks b with dense weights W_b (a block-diagonal W), Z
the standardised genotypes of the streamer.  One application is two passes
over the packed genotypes on the tensor cores plus one batched FP32 GEMM:

    T = Z^T V             coherit_geno_xtv   (m x k)
    S_b = W_b T_b / c     torch.bmm over W buckets resident in HBM
    K V = Z S             coherit_geno_zxb   (n x k)

The normaliser c is the kernel trace sum_b tr(Z_b W_b Z_b^T)/n
(smile_block_w.py:692-726) or the sum of the blocks' effective ranks; the
per-block traces and the per-sample diagonal are computed once from
standardised genotype columns extracted on the device.  Names, arguments and
errors follow the reference module.
"""
from __future__ import annotations

import dataclasses
import json
import os
import shutil
import subprocess
import tempfile
from pathlib import Path
from typing import Literal, Sequence

import numpy as np
import torch

from .geno_stream import as_rhs

Normalization = Literal["kernel_trace", "effective_rank"]
DiagMode = Literal["full", "mean"]
_VALID_NORMALIZATIONS = ("kernel_trace", "effective_rank")
_EFFECTIVE_RANK_KEYS = ("effective_rank", "retained_rank", "weight_rank", "rank")
_IDENTITY_TRACE_SCAN_TARGET_BYTES = 256 * 1024 * 1024
_W_DEVICE_CACHE_CAP_BYTES = 8 * 1024**3
_W_DEVICE_CACHE_FRACTION = 0.35
_W_BUCKET_WIDTH_MULTIPLE = 512
_W_BUCKET_LOCAL_TARGET_BYTES = 4 * 1024**3
_W_BUCKET_ASSUMED_RHS = 1024


@dataclasses.dataclass(frozen=True)
class SmileBlockWeight:
    """A single contiguous block W_i in cache order (smile_block_w.py:44-62)."""

    matrix: np.ndarray | None
    start: int
    size_value: int
    trace_per_sample: float
    source: str | None = None
    is_identity: bool = False
    device_matrix: object | None = None

    @property
    def size(self) -> int:
        return int(self.size_value)

    @property
    def stop(self) -> int:
        return int(self.start + self.size)


@dataclasses.dataclass(frozen=True)
class SmileBlockBucket:
    """W blocks of one padded width, stacked for one batched GEMM.

    ``matrices`` (B, w, w) FP32 zero-padded; ``index`` (B, w) SNP rows of
    each block (padding rows point at row 0 and are masked by ``mask``)."""

    matrices: torch.Tensor
    index: torch.Tensor
    mask: torch.Tensor
    starts: np.ndarray
    sizes: np.ndarray
    width: int


def default_w_device_cache_bytes(gpu_budget_bytes: float | None) -> float:
    """Default dense-W device cache limit (smile_block_w.py:74-82)."""
    if gpu_budget_bytes is None:
        return 0.0
    budget = float(gpu_budget_bytes)
    if not np.isfinite(budget) or budget <= 0.0:
        return 0.0
    return float(min(_W_DEVICE_CACHE_CAP_BYTES, _W_DEVICE_CACHE_FRACTION * budget))


def _bucket_width(width: int) -> int:
    multiple = int(_W_BUCKET_WIDTH_MULTIPLE)
    return int(((int(width) + multiple - 1) // multiple) * multiple)


def estimate_bucketed_w_device_cache_bytes(widths: Sequence[int],
                                           cache_limit_bytes: float | None) -> float:
    """Padded bucket bytes if the W blocks fit the limit, else 0."""
    limit = float(cache_limit_bytes or 0.0)
    if limit <= 0.0:
        return 0.0
    padded = float(sum(_bucket_width(int(w)) ** 2 * 4 for w in widths))
    return padded if 0.0 < padded <= limit else 0.0


def estimate_bucketed_w_local_workspace_bytes(widths: Sequence[int], *,
                                              rhs_cols: int = _W_BUCKET_ASSUMED_RHS,
                                              cache_enabled: bool) -> float:
    """Conservative local + output workspace of the bucketed W products."""
    if not cache_enabled:
        return 0.0
    groups: dict[int, int] = {}
    for w in widths:
        bw = _bucket_width(int(w))
        groups[bw] = groups.get(bw, 0) + 1
    max_local = 0.0
    for bw, count in groups.items():
        max_blocks = max(1, int(_W_BUCKET_LOCAL_TARGET_BYTES // (bw * int(rhs_cols) * 4)))
        max_local = max(max_local, float(min(count, max_blocks) * bw * int(rhs_cols) * 4))
    return 2.0 * max_local


# ------------------------------------------------------------------ W files

def load_rds_matrix(path: str | os.PathLike[str]) -> np.ndarray:
    """Numeric matrix from an R ``.rds`` file, converted through ``Rscript``."""
    rscript = shutil.which("Rscript")
    if rscript is None:
        raise RuntimeError("Reading .rds weight files needs Rscript on PATH.")
    code = ("a <- commandArgs(trailingOnly=TRUE); x <- as.matrix(readRDS(a[1])); "
            "storage.mode(x) <- 'double'; con <- file(a[2], 'wb'); "
            "writeBin(as.integer(dim(x)), con, size=4); writeBin(as.vector(t(x)), con, size=8); "
            "close(con)")
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "w.bin")
        subprocess.run([rscript, "-e", code, os.fspath(path), out], check=True,
                       capture_output=True)
        raw = Path(out).read_bytes()
    rows, cols = np.frombuffer(raw[:8], dtype="<i4")
    return np.frombuffer(raw[8:], dtype="<f8").reshape(int(rows), int(cols)).copy()


def load_weight_matrix(path: str | os.PathLike[str]) -> np.ndarray:
    """Dense W from .rds, .npy/.npz or text/CSV (smile_block_w.py:180-199)."""
    path = Path(path)
    suffix = path.suffix.lower()
    if suffix == ".rds":
        return load_rds_matrix(path)
    if suffix == ".npy":
        return np.load(path, mmap_mode="r")
    if suffix == ".npz":
        with np.load(path) as data:
            keys = list(data.files)
            if len(keys) != 1:
                raise ValueError(f"NPZ weight file must contain exactly one array, got {keys}.")
            return data[keys[0]]
    return np.loadtxt(path, delimiter="," if suffix == ".csv" else None)


def load_weight_matrix_metadata(path: str | os.PathLike[str], *, required: bool = False) -> dict:
    """Sidecar JSON next to a W file (``.json`` or ``.meta.json``)."""
    matrix_path = Path(path)
    candidates = (matrix_path.with_suffix(".json"), matrix_path.with_suffix(".meta.json"))
    meta_path = next((c for c in candidates if c.exists()), None)
    if meta_path is None:
        if required:
            raise ValueError(
                f"Missing sidecar JSON metadata for W file {os.fspath(path)!r}; looked for "
                + ", ".join(os.fspath(c) for c in candidates) + ".")
        return {}
    try:
        meta = json.loads(meta_path.read_text())
    except (OSError, json.JSONDecodeError) as exc:
        if required:
            raise ValueError(f"Failed to read sidecar JSON metadata {os.fspath(meta_path)!r}.") from exc
        return {}
    if not isinstance(meta, dict):
        raise ValueError(f"Sidecar JSON metadata must be an object: {os.fspath(meta_path)!r}.")
    return meta


def load_weight_matrix_shape(path: str | os.PathLike[str]) -> tuple[int, int]:
    """W shape from sidecar metadata or the file header when possible."""
    path = Path(path)
    meta = load_weight_matrix_metadata(path, required=False)
    for key in ("shape", "matrix_shape"):
        if key in meta:
            shape = tuple(int(x) for x in meta[key])
            if len(shape) == 2:
                return shape
    for key in ("width", "size", "p", "n_snps"):
        if key in meta:
            return (int(meta[key]), int(meta[key]))
    suffix = path.suffix.lower()
    if suffix == ".npy":
        return tuple(int(x) for x in np.load(path, mmap_mode="r").shape)
    return tuple(int(x) for x in np.asarray(load_weight_matrix(path)).shape)


def validate_weight_matrix(matrix: np.ndarray, *, name: str = "W") -> np.ndarray:
    """Finite square FP32 W (smile_block_w.py:267-288)."""
    arr = np.asarray(matrix)
    if arr.ndim != 2 or arr.shape[0] != arr.shape[1]:
        raise ValueError(f"{name} must be a square matrix, got shape {arr.shape}.")
    if arr.shape[0] == 0:
        raise ValueError(f"{name} must be non-empty.")
    if not np.issubdtype(arr.dtype, np.number):
        raise ValueError(f"{name} must be numeric, got dtype={arr.dtype}.")
    W = np.ascontiguousarray(arr, dtype=np.float32)
    if not np.all(np.isfinite(W)):
        raise ValueError(f"{name} contains non-finite values.")
    return W


# ---------------------------------------------------------------- operator

def _diag_of_block(streamer, W: np.ndarray | None, start: int, size: int) -> torch.Tensor:
    """diag(Z_b W_b Z_b^T) per sample (FP64), Z_b extracted on the device;
    FP32 products as in the reference (smile_block_w.py:669-689)."""
    Z = streamer.standardized_columns(np.arange(start, start + size))
    if W is None:
        return torch.sum((Z * Z).double(), dim=1)
    Wd = torch.as_tensor(W, dtype=torch.float32, device=streamer.dev)
    return torch.sum((torch.matmul(Z, Wd) * Z).double(), dim=1)


def _build_buckets(blocks: Sequence[SmileBlockWeight], dev) -> tuple[SmileBlockBucket, ...]:
    groups: dict[int, list[SmileBlockWeight]] = {}
    for blk in blocks:
        if blk.is_identity or blk.matrix is None:
            continue
        groups.setdefault(_bucket_width(blk.size), []).append(blk)
    buckets = []
    for width in sorted(groups):
        group = groups[width]
        W = np.zeros((len(group), width, width), dtype=np.float32)
        index = np.zeros((len(group), width), dtype=np.int64)
        mask = np.zeros((len(group), width), dtype=np.float32)
        for b, blk in enumerate(group):
            W[b, :blk.size, :blk.size] = blk.matrix
            index[b, :blk.size] = np.arange(blk.start, blk.stop)
            mask[b, :blk.size] = 1.0
        buckets.append(SmileBlockBucket(
            matrices=torch.as_tensor(W, device=dev), index=torch.as_tensor(index, device=dev),
            mask=torch.as_tensor(mask, device=dev),
            starts=np.asarray([b.start for b in group], dtype=np.int64),
            sizes=np.asarray([b.size for b in group], dtype=np.int64), width=width))
    return tuple(buckets)


class SmileBlockWeightedOperator:
    """Matrix-free SMILE block-diagonal W operator over a GenoBlockStreamer
    (smile_block_w.py:390-949)."""

    def __init__(self, streamer, weight_matrices: Sequence[np.ndarray], *,
                 normalization: Normalization = "kernel_trace", strict_coverage: bool = True,
                 sources: Sequence[str | None] | None = None,
                 start_offsets: Sequence[int] | None = None,
                 effective_ranks: Sequence[float] | None = None, diag_mode: DiagMode = "full",
                 device_cache_max_bytes: float | None = None):
        if normalization not in _VALID_NORMALIZATIONS:
            raise ValueError(f"normalization must be one of {_VALID_NORMALIZATIONS}.")
        if diag_mode not in ("full", "mean"):
            raise ValueError("diag_mode must be 'full' or 'mean'.")
        if not weight_matrices:
            raise ValueError("At least one weight matrix is required.")
        for name, seq in (("sources", sources), ("start_offsets", start_offsets),
                          ("effective_ranks", effective_ranks)):
            if seq is not None and len(seq) != len(weight_matrices):
                raise ValueError(f"{name} length must match weight_matrices length.")
        n = int(streamer.n)
        raw_diag = torch.zeros(n, dtype=torch.float64, device=streamer.dev) \
            if diag_mode == "full" else None
        raw_trace = 0.0
        blocks = []
        next_start = 0
        for idx, raw_W in enumerate(weight_matrices):
            source = None if sources is None else sources[idx]
            W = validate_weight_matrix(raw_W, name=f"W[{idx}]")
            start = int(start_offsets[idx]) if start_offsets is not None else int(next_start)
            if start < 0:
                raise ValueError(f"W[{idx}] start offset must be non-negative, got {start}.")
            stop = start + int(W.shape[0])
            if stop > int(streamer.m):
                raise ValueError(f"W[{idx}] with size {W.shape[0]} exceeds streamer.m={int(streamer.m)}.")
            contrib = _diag_of_block(streamer, W, start, int(W.shape[0]))
            kernel_trace = float(contrib.sum()) / n
            if raw_diag is not None:
                raw_diag += contrib
            elif not np.isfinite(kernel_trace) or kernel_trace <= 0.0:
                raise ValueError(f"Invalid SMILE block trace contribution: {kernel_trace!r}.")
            if normalization == "effective_rank":
                trace_per_sample = self._effective_rank_contribution(
                    source=source,
                    explicit_rank=None if effective_ranks is None else effective_ranks[idx],
                    width=int(W.shape[0]), block_name=f"W[{idx}]")
            else:
                trace_per_sample = kernel_trace
            raw_trace += kernel_trace
            blocks.append(SmileBlockWeight(matrix=W, start=start, size_value=int(W.shape[0]),
                                           trace_per_sample=trace_per_sample, source=source))
            next_start = stop
        if strict_coverage and start_offsets is None and next_start != int(streamer.m):
            raise ValueError(
                f"Block W matrices cover {next_start} SNPs but streamer.m={int(streamer.m)}. "
                "Pass strict_coverage=False to intentionally ignore trailing SNPs.")
        self._finish(streamer, blocks, normalization, diag_mode, strict_coverage, raw_diag,
                     raw_trace)

    def _finish(self, streamer, blocks, normalization, diag_mode, strict_coverage, raw_diag,
                raw_trace):
        self.streamer = streamer
        self.blocks = tuple(blocks)
        self.normalization = normalization
        self.normalizer = self._compute_global_normalizer(
            [b.trace_per_sample for b in blocks], normalization=normalization)
        self._buckets = _build_buckets(self.blocks, streamer.dev)
        id_rows = [np.arange(b.start, b.stop) for b in self.blocks if b.is_identity]
        self._identity_rows = (torch.as_tensor(np.concatenate(id_rows), device=streamer.dev)
                               if id_rows else None)
        self.w_device_cache_bytes = float(sum(b.matrices.numel() * 4 for b in self._buckets))
        if raw_diag is None:
            self._diag_dev = torch.tensor(raw_trace / self.normalizer, dtype=torch.float32,
                                          device=streamer.dev)
        else:
            self._diag_dev = (raw_diag / self.normalizer).float()
        self._diag_host = self._diag_dev.cpu().numpy()
        self.strict_coverage = bool(strict_coverage)
        self.diag_mode = diag_mode

    @classmethod
    def identity(cls, streamer, *, block_size: int | None = None,
                 normalization: Normalization = "kernel_trace", strict_coverage: bool = True,
                 diag_mode: DiagMode = "full") -> "SmileBlockWeightedOperator":
        """The operator for W = I without materialising I (smile_block_w.py:518-605)."""
        if normalization not in _VALID_NORMALIZATIONS:
            raise ValueError(f"normalization must be one of {_VALID_NORMALIZATIONS}.")
        if diag_mode not in ("full", "mean"):
            raise ValueError("diag_mode must be 'full' or 'mean'.")
        if block_size is None:
            block_size = cls._auto_identity_block_size(streamer, normalization=normalization)
        block_size = int(block_size)
        if block_size <= 0:
            raise ValueError("block_size must be positive.")
        if int(streamer.m) <= 0:
            raise ValueError("streamer must contain at least one SNP.")
        n = int(streamer.n)
        raw_diag = torch.zeros(n, dtype=torch.float64, device=streamer.dev) \
            if diag_mode == "full" else None
        raw_trace = 0.0
        blocks = []
        start = 0
        while start < int(streamer.m):
            size = min(block_size, int(streamer.m) - start)
            contrib = _diag_of_block(streamer, None, start, size)
            kernel_trace = float(contrib.sum()) / n
            if raw_diag is not None:
                raw_diag += contrib
            elif not np.isfinite(kernel_trace) or kernel_trace <= 0.0:
                raise ValueError(f"Invalid SMILE block trace contribution: {kernel_trace!r}.")
            raw_trace += kernel_trace
            tps = float(size) if normalization == "effective_rank" else kernel_trace
            blocks.append(SmileBlockWeight(matrix=None, start=start, size_value=size,
                                           trace_per_sample=tps, source="identity",
                                           is_identity=True))
            start += size
        self = cls.__new__(cls)
        self._finish(streamer, blocks, normalization, diag_mode, strict_coverage, raw_diag,
                     raw_trace)
        return self

    @staticmethod
    def _auto_identity_block_size(streamer, *, normalization: Normalization) -> int:
        width = int(_IDENTITY_TRACE_SCAN_TARGET_BYTES // (max(1, int(streamer.n)) * 4))
        return int(min(int(streamer.m), max(1, width)))

    @classmethod
    def from_weight_files(cls, streamer, paths: Sequence[str | os.PathLike[str]], **kwargs):
        matrices = [load_weight_matrix(p) for p in paths]
        return cls(streamer, matrices, sources=[os.fspath(p) for p in paths], **kwargs)

    @staticmethod
    def _effective_rank_contribution(*, source, explicit_rank, width: int, block_name: str) -> float:
        if explicit_rank is None:
            if source is None:
                raise ValueError(
                    f"{block_name} uses effective_rank normalization but has no sidecar "
                    "metadata or explicit effective rank.")
            meta = load_weight_matrix_metadata(source, required=True)
            for key in _EFFECTIVE_RANK_KEYS:
                if key in meta:
                    explicit_rank = meta[key]
                    break
            else:
                raise ValueError(
                    f"{block_name} sidecar metadata for effective_rank normalization must "
                    f"contain one of {_EFFECTIVE_RANK_KEYS}.")
        value = float(explicit_rank)
        if not np.isfinite(value) or value <= 0.0:
            raise ValueError(f"Invalid effective rank for {block_name}: {explicit_rank!r}.")
        if value > float(width) * (1.0 + 1e-6):
            raise ValueError(
                f"Invalid effective rank for {block_name}: {value:g} exceeds block width {width}.")
        return value

    @staticmethod
    def _compute_global_normalizer(trace_values: Sequence[float], *,
                                   normalization: Normalization) -> float:
        value = float(np.sum(np.asarray(trace_values, dtype=np.float64)))
        if not np.isfinite(value) or value <= 0.0:
            raise ValueError(f"Invalid SMILE global normalizer: {value!r}.")
        return value

    # ------------------------------------------------------------ products
    @property
    def n_blocks(self) -> int:
        return len(self.blocks)

    def diag(self) -> torch.Tensor:
        """Per-sample diagonal (``diag_mode="full"``) or the scalar mean."""
        return self._diag_dev

    def _accumulate_weighted_scores_from_xtv(self, scores: torch.Tensor, XtV: torch.Tensor, *,
                                             scale=1.0, block_idx: int | None = None):
        """scores[b rows] += scale/c * W_b XtV[b rows] (smile_block_w.py:786-829)."""
        f = float(scale) / float(self.normalizer)
        if block_idx is None:
            for bk in self._buckets:
                local = XtV[bk.index] * bk.mask[:, :, None]                  # (B, w, k)
                weighted = torch.bmm(bk.matrices, local) * bk.mask[:, :, None]
                scores.index_add_(0, bk.index.reshape(-1),
                                  (weighted * f).reshape(-1, XtV.shape[1]))
            if self._identity_rows is not None:
                scores.index_add_(0, self._identity_rows, f * XtV[self._identity_rows])
            return scores
        blk = self.blocks[int(block_idx)]
        local = XtV[blk.start:blk.stop]
        if not blk.is_identity:
            Wd = torch.as_tensor(blk.matrix, device=XtV.device)
            local = Wd @ local
        scores[blk.start:blk.stop] += f * local
        return scores

    def _weighted_scores(self, V: torch.Tensor, block_idx: int | None = None) -> torch.Tensor:
        XtV = self.streamer.xtv(V, normalize=False)
        if XtV.ndim == 1:
            XtV = XtV[:, None]
        scores = torch.zeros((int(self.streamer.m), XtV.shape[1]), dtype=torch.float32,
                             device=XtV.device)
        return self._accumulate_weighted_scores_from_xtv(scores, XtV, block_idx=block_idx)

    def kv(self, V) -> torch.Tensor:
        """``sum_b Z_b W_b Z_b^T V / c``."""
        Vm, squeeze = as_rhs(V, self.streamer.dev)
        out = self.streamer.zxb(self._weighted_scores(Vm))
        return out[:, 0] if squeeze else out

    def block_kv(self, V, block_idx: int) -> torch.Tensor:
        """One block's contribution ``Z_b W_b Z_b^T V / c``."""
        if block_idx < 0 or block_idx >= len(self.blocks):
            raise IndexError(f"block_idx={block_idx} out of range for {len(self.blocks)} blocks.")
        Vm, squeeze = as_rhs(V, self.streamer.dev)
        out = self.streamer.zxb(self._weighted_scores(Vm, block_idx=block_idx))
        return out[:, 0] if squeeze else out

    def stacked_block_kv(self, V) -> torch.Tensor:
        return torch.stack([self.block_kv(V, i) for i in range(len(self.blocks))], dim=0)

    def weighted_hv(self, theta_g, theta_e, V) -> torch.Tensor:
        """``theta_e V + theta_g K V`` with one genetic component."""
        tg = np.asarray(theta_g, dtype=np.float64)
        if tg.ndim == 1 and tg.size == 1:
            tg = tg[0]
        elif tg.ndim != 0:
            raise ValueError("theta_g must be a scalar or a length-one array for SMILE block-W.")
        Vm, squeeze = as_rhs(V, self.streamer.dev)
        XtV = self.streamer.xtv(Vm, normalize=False)
        scores = torch.zeros((int(self.streamer.m), Vm.shape[1]), dtype=torch.float32,
                             device=Vm.device)
        scores = self._accumulate_weighted_scores_from_xtv(scores, XtV, scale=float(tg))
        out = self.streamer.zxb(scores)
        if theta_e is not None:
            out = out + float(np.asarray(theta_e).reshape(-1)[0]) * Vm
        return out[:, 0] if squeeze else out

    def snp_effects(self, alpha, theta_g) -> torch.Tensor:
        """beta with ``Z beta = theta_g K alpha``: theta_g/c W_b Z_b^T alpha."""
        tg = np.asarray(theta_g, dtype=np.float64)
        if tg.ndim == 1 and tg.size == 1:
            tg = tg[0]
        elif tg.ndim != 0:
            raise ValueError("theta_g must be a scalar or a length-one array for SMILE block-W.")
        a, squeeze = as_rhs(alpha, self.streamer.dev)
        if a.shape[1] != 1:
            raise ValueError("snp_effects expects a single alpha vector.")
        XtA = self.streamer.xtv(a, normalize=False)
        beta = torch.zeros((int(self.streamer.m), 1), dtype=torch.float32, device=a.device)
        beta = self._accumulate_weighted_scores_from_xtv(beta, XtA, scale=float(tg))
        return beta[:, 0]


class SmileMultiBlockWeightedOperator:
    """Several SMILE GRMs (variance components) sharing one streamer
    (smile_block_w.py:952-1127); one X^T V pass serves all of them."""

    def __init__(self, operators: Sequence[SmileBlockWeightedOperator]):
        if not operators:
            raise ValueError("At least one SMILE operator is required.")
        streamer = operators[0].streamer
        for idx, op in enumerate(operators):
            if op.streamer is not streamer:
                raise ValueError(f"SMILE operator {idx} uses a different streamer.")
        self.streamer = streamer
        self.operators = tuple(operators)

    @classmethod
    def from_weight_matrix_groups(cls, streamer, weight_matrix_groups, *,
                                  normalization: Normalization = "kernel_trace",
                                  strict_coverage: bool = True, source_groups=None,
                                  effective_rank_groups=None, diag_mode: DiagMode = "full",
                                  device_cache_max_bytes: float | None = None):
        groups = [list(g) for g in weight_matrix_groups]
        if not groups or any(len(g) == 0 for g in groups):
            raise ValueError("SMILE GRM groups must be non-empty.")
        if source_groups is not None and len(source_groups) != len(groups):
            raise ValueError("source_groups length must match weight_matrix_groups length.")
        if effective_rank_groups is not None and len(effective_rank_groups) != len(groups):
            raise ValueError("effective_rank_groups length must match weight_matrix_groups length.")
        operators = []
        next_start = 0
        for gi, group in enumerate(groups):
            starts = []
            for matrix in group:
                arr = np.asarray(matrix)
                if arr.ndim != 2 or arr.shape[0] != arr.shape[1]:
                    raise ValueError(
                        f"W group {gi} contains a non-square matrix with shape {arr.shape}.")
                starts.append(next_start)
                next_start += int(arr.shape[0])
            ranks = None if effective_rank_groups is None else list(effective_rank_groups[gi])
            if ranks is not None and len(ranks) != len(group):
                raise ValueError(f"effective_rank_groups[{gi}] length must match W group length.")
            operators.append(SmileBlockWeightedOperator(
                streamer, group, normalization=normalization, strict_coverage=False,
                sources=None if source_groups is None else list(source_groups[gi]),
                start_offsets=starts, effective_ranks=ranks, diag_mode=diag_mode))
        if strict_coverage and next_start != int(streamer.m):
            raise ValueError(
                f"SMILE GRM groups cover {next_start} SNPs but streamer.m={int(streamer.m)}. "
                "Pass strict_coverage=False to intentionally ignore trailing SNPs.")
        return cls(operators)

    @classmethod
    def from_weight_file_groups(cls, streamer, path_groups, **kwargs):
        matrix_groups = [[load_weight_matrix(p) for p in g] for g in path_groups]
        source_groups = [[os.fspath(p) for p in g] for g in path_groups]
        return cls.from_weight_matrix_groups(streamer, matrix_groups,
                                             source_groups=source_groups, **kwargs)

    @property
    def n_grm(self) -> int:
        return len(self.operators)

    def diag_list(self) -> tuple:
        return tuple(op.diag() for op in self.operators)

    def kv(self, V, grm_idx: int) -> torch.Tensor:
        return self.operators[int(grm_idx)].kv(V)

    def stacked_kv(self, V) -> torch.Tensor:
        Vm, squeeze = as_rhs(V, self.streamer.dev)
        XtV = self.streamer.xtv(Vm, normalize=False)
        outs = []
        for op in self.operators:
            scores = torch.zeros((int(self.streamer.m), Vm.shape[1]), dtype=torch.float32,
                                 device=Vm.device)
            out = self.streamer.zxb(op._accumulate_weighted_scores_from_xtv(scores, XtV))
            outs.append(out[:, 0] if squeeze else out)
        return torch.stack(outs, dim=0)

    def weighted_hv(self, theta_g, theta_e, V) -> torch.Tensor:
        tg = np.asarray(theta_g, dtype=np.float64).reshape(-1)
        if tg.size != len(self.operators):
            raise ValueError(
                f"theta_g must be a length-{len(self.operators)} array for SMILE multi-GRM.")
        Vm, squeeze = as_rhs(V, self.streamer.dev)
        XtV = self.streamer.xtv(Vm, normalize=False)
        scores = torch.zeros((int(self.streamer.m), Vm.shape[1]), dtype=torch.float32,
                             device=Vm.device)
        for i, op in enumerate(self.operators):
            scores = op._accumulate_weighted_scores_from_xtv(scores, XtV, scale=float(tg[i]))
        out = self.streamer.zxb(scores)
        if theta_e is not None:
            out = out + float(np.asarray(theta_e).reshape(-1)[0]) * Vm
        return out[:, 0] if squeeze else out

    def snp_effects(self, alpha, theta_g) -> tuple:
        tg = np.asarray(theta_g, dtype=np.float64).reshape(-1)
        if tg.size != len(self.operators):
            raise ValueError(
                f"theta_g must be a length-{len(self.operators)} array for SMILE multi-GRM.")
        return tuple(op.snp_effects(alpha, tg[i]) for i, op in enumerate(self.operators))


__all__ = [
    "SmileBlockWeight", "SmileBlockBucket", "SmileBlockWeightedOperator",
    "SmileMultiBlockWeightedOperator", "default_w_device_cache_bytes",
    "estimate_bucketed_w_device_cache_bytes", "estimate_bucketed_w_local_workspace_bytes",
    "load_rds_matrix", "load_weight_matrix", "load_weight_matrix_metadata",
    "load_weight_matrix_shape", "validate_weight_matrix",
]
