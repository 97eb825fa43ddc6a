"""Resident genotype "streamer" with the reference's call surface.

``GenoBlockStreamer`` mirrors GPU_REML's streamer (geno_stream.py:1147-2864):
same constructor arguments, call geometry, per-SNP statistics, attributes
and operator methods.  Instead of a host tmpfile cache streamed over PCIe per
operator application (geno_stream.py:2358-2396, kv_impl.py:300-320), the
2-bit genotypes are transcoded once into HBM-resident layouts owned by the
CUDA library, and every method below is one or two kernel launches on the
caller's current CUDA stream.

Tensors are ``torch`` CUDA tensors (float32 right-hand sides, row-major).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Sequence

import numpy as np
import torch

from . import _lib
from .block_backend import DensePackedBlockDescriptor

_DEFAULT_PRECISION = os.environ.get("COHERIT_PRECISION", "bf16x3")


# --------------------------------------------------------------- sources

class ArraySource:
    """In-memory genotype source: (n, m) int8/uint8 allele counts.

    ``read_block_variant_major(start, count)`` returns a (count, n) int8
    block like the reference's sources (geno_stream.py:2576-2599).
    """

    def __init__(self, genotypes: np.ndarray, missing_val: int = -127, sample_ids=None):
        g = np.asarray(genotypes)
        if g.ndim != 2:
            raise ValueError("genotypes must be a 2-D (samples, variants) array")
        self._g = g
        self.n = int(g.shape[0])
        self.m = int(g.shape[1])
        self.missing_val = int(missing_val)
        self.sample_ids = sample_ids

    def read_block_variant_major(self, start: int, count: int) -> np.ndarray:
        blk = np.ascontiguousarray(self._g[:, start:start + count].T)
        return blk.astype(np.int8) if blk.dtype != np.int8 else blk


class SyntheticSource:
    """Generator-backed source: Binomial(2, MAF) genotypes, MAF ~ U(0.05, 0.5).

    The streamer builds its resident matrix directly on the device from the
    same counter-based hash (no host copy of the genotypes).
    """

    def __init__(self, n: int, m: int, seed: int = 0, missing_rate: float = 0.0):
        from .synth import missing_rate_q24

        self.n = int(n)
        self.m = int(m)
        self.seed = int(seed)
        self.missing_q24 = missing_rate_q24(missing_rate)
        self.missing_val = -127
        self.sample_ids = None

    def read_block_variant_major(self, start: int, count: int) -> np.ndarray:
        from .synth import genotype_codes

        codes = genotype_codes(self.seed, self.n, np.arange(start, start + count), self.missing_q24)
        out = codes.T.astype(np.int8)
        out[codes.T == 3] = self.missing_val
        return out


class LDBlockSource:
    """Generator-backed source with linkage disequilibrium (synth.ld_tables):
    SNPs in blocks of ``block`` with AR(1) latent haplotypes, rho ~
    U(rho_range), MAF ~ U(0.05, 0.5).  The streamer builds its resident
    matrix on the device (coherit_geno_create_ldblock); host reads give the
    same codes from the numpy twin (small sizes)."""

    def __init__(self, n: int, m: int, seed: int = 0, block: int = 200, rho_range=(0.0, 0.9)):
        from .synth import ld_tables

        self.n = int(n)
        self.m = int(m)
        self.seed = int(seed)
        self.block = int(block)
        self.tables = ld_tables(self.seed, self.m, block=self.block, rho_range=rho_range)
        self.missing_val = -127
        self.sample_ids = None

    def read_block_variant_major(self, start: int, count: int) -> np.ndarray:
        from .synth import ld_block_codes

        if start % self.block:
            raise ValueError("host reads of the LD-block source start on a block boundary")
        codes = ld_block_codes(self.seed, self.n, self.m, block=self.block, tables=self.tables)
        return np.ascontiguousarray(codes[:, start:start + count].T.astype(np.int8))


def _normalize_component_block_sizes(m: int, component_block_sizes) -> list[int]:
    """Contiguous component sizes: positive, summing to m (geno_stream.py:371-392)."""
    if component_block_sizes is None:
        return [int(m)]
    sizes = np.asarray(component_block_sizes, dtype=np.int64).reshape(-1)
    if sizes.size == 0:
        raise ValueError("component_block_sizes must contain at least one block.")
    if np.any(sizes <= 0):
        raise ValueError("component_block_sizes must be strictly positive.")
    total = int(np.sum(sizes))
    if total != int(m):
        raise ValueError(f"component_block_sizes must sum to m={int(m)}; got {total}.")
    return [int(x) for x in sizes.tolist()]


def _normalize_component_variant_indices(m: int, component_variant_indices):
    """Arbitrary variant groups -> (sizes, cache_to_source) (geno_stream.py:395-437).

    Each group is sorted, so the SNPs of a component sit in source order in
    the cache; groups must be disjoint, free of duplicates and inside [0, m).
    A group without SNPs is rejected (the reference accepts it as an empty
    component).
    """
    groups = list(component_variant_indices or [])
    if not groups:
        raise ValueError("component_variant_indices must contain at least one component.")
    normalized = []
    for comp_idx, group in enumerate(groups):
        arr = np.asarray(group, dtype=np.int64).reshape(-1)
        if arr.size == 0:
            raise ValueError(f"component_variant_indices[{comp_idx}] is empty; every "
                             "component needs at least one SNP.")
        if np.any((arr < 0) | (arr >= int(m))):
            raise IndexError(f"component_variant_indices[{comp_idx}] contains out-of-range "
                             f"SNP indices for m={int(m)}.")
        uniq = np.unique(arr)
        if uniq.size != arr.size:
            raise ValueError(f"component_variant_indices[{comp_idx}] contains duplicate SNP "
                             "indices.")
        normalized.append(uniq)
    cache_to_source = np.concatenate(normalized)
    if cache_to_source.size > int(m):
        raise ValueError(f"component_variant_indices assign {cache_to_source.size} SNPs, "
                         f"which exceeds source m={int(m)}.")
    if np.unique(cache_to_source).size != cache_to_source.size:
        raise ValueError("component_variant_indices must be disjoint across components.")
    return [int(g.size) for g in normalized], cache_to_source


def _build_call_geometry(m: int, call_width: int, component_sizes: Sequence[int]):
    """Call blocks of width <= call_width inside each component (geno_stream.py:469-505)."""
    starts, widths, comps, offsets = [], [], [], [0]
    pos = 0
    for g, size in enumerate(component_sizes):
        left = int(size)
        while left > 0:
            w = min(int(call_width), left)
            starts.append(pos)
            widths.append(w)
            comps.append(g)
            pos += w
            left -= w
        offsets.append(len(starts))
    return (
        np.asarray(starts, dtype=np.int64),
        np.asarray(widths, dtype=np.int32),
        np.asarray(comps, dtype=np.int32),
        np.asarray(offsets, dtype=np.int32),
    )


def _pack_lut(missing_val: int) -> np.ndarray:
    lut = np.zeros(256, dtype=np.uint8)
    lut[1] = 1
    lut[2] = 2
    lut[int(np.asarray([missing_val], dtype=np.int8).view(np.uint8)[0])] = 3
    return lut


def _pack_block_vm(block_vm: np.ndarray, lut: np.ndarray) -> np.ndarray:
    """(w, n) int8 variant-major -> (n, ceil(w/4)) packed codes."""
    codes = lut[np.asarray(block_vm).view(np.uint8)].T  # (n, w)
    n, w = codes.shape
    pw = (w + 3) // 4
    pad = np.zeros((n, 4 * pw), dtype=np.uint8)
    pad[:, :w] = codes
    q = pad.reshape(n, pw, 4)
    return (q[:, :, 0] | (q[:, :, 1] << 2) | (q[:, :, 2] << 4) | (q[:, :, 3] << 6)).astype(np.uint8)


def _device_of(device) -> torch.device:
    if device is None or device == "auto":
        if not torch.cuda.is_available():
            raise RuntimeError("coherit_gb300 requires a CUDA device (no CPU fallback)")
        return torch.device("cuda", torch.cuda.current_device())
    dev = torch.device(device)
    if dev.type != "cuda":
        raise RuntimeError(f"coherit_gb300 operators run on CUDA devices only, got {dev}")
    return dev


def as_rhs(V, device: torch.device) -> tuple[torch.Tensor, bool]:
    """Right-hand side as a contiguous float32 (n, k) CUDA tensor."""
    if not isinstance(V, torch.Tensor):
        V = torch.as_tensor(np.asarray(V, dtype=np.float32))
    squeeze = V.ndim == 1
    if squeeze:
        V = V[:, None]
    if V.ndim != 2:
        raise ValueError(f"right-hand side must be 1-D or 2-D, got shape {tuple(V.shape)}")
    V = V.to(device=device, dtype=torch.float32)
    if not V.is_contiguous():
        V = V.contiguous()
    return V, squeeze


class GenoBlockStreamer:
    """HBM-resident genotype operator with GPU_REML's streamer interface."""

    def __init__(
        self,
        source=None,
        *,
        bed_prefix: str | None = None,
        call_width: int = 131072,
        component_block_sizes=None,
        component_variant_indices=None,
        standardization_override: tuple[np.ndarray, np.ndarray] | None = None,
        device=None,
        keep_host_stats: bool = True,
        build_threads: int | None = None,
        sample_mask: np.ndarray | None = None,
        ring_depth: int | None = None,
        source_build_chunk_width: int | None = None,
        precision: str | None = None,
    ):
        if source is not None and bed_prefix is not None:
            raise ValueError("Provide either source or bed_prefix, not both.")
        if source is None:
            if bed_prefix is None:
                raise ValueError("Either source or bed_prefix must be provided.")
            from .bed import BedSource

            source = BedSource(bed_prefix)
        self._lib = _lib.load()
        self.dev = _device_of(device)
        self.precision = precision or _DEFAULT_PRECISION
        if self.precision not in _lib.PRECISIONS:
            raise ValueError(f"unknown precision {self.precision!r}")
        self._prec = _lib.PRECISIONS[self.precision]
        self.keep_host_stats = bool(keep_host_stats)
        self.bed_prefix = bed_prefix
        self._source_n = int(source.n)
        self.source_m = int(source.m)
        self._sample_mask = None if sample_mask is None else np.asarray(sample_mask, dtype=bool)
        if self._sample_mask is not None and self._sample_mask.shape != (self._source_n,):
            raise ValueError(
                "sample_mask is incompatible with the supplied source: "
                f"mask length={self._sample_mask.size}, "
                f"selected={int(np.count_nonzero(self._sample_mask))}, source.n={self._source_n}."
            )
        # The reference sizes its host ring with ring_depth (geno_stream.py:171-173);
        # the resident operator has no ring, but the argument is checked alike.
        if ring_depth is not None and int(ring_depth) <= 0:
            raise ValueError("ring depth must be positive when provided.")
        self.n = int(self._sample_mask.sum()) if self._sample_mask is not None else self._source_n
        if self.n <= 0:
            raise ValueError("Genotype source must contain at least one selected sample.")
        if self.source_m <= 0:
            raise ValueError("Genotype source must contain at least one variant.")
        sample_ids = getattr(source, "sample_ids", None)
        self.sample_ids = (
            None if sample_ids is None else
            tuple(s for s, k in zip(sample_ids, self._sample_mask) if k) if self._sample_mask is not None
            else tuple(sample_ids)
        )
        self._missing_val = np.uint8(3)
        self.call_width = max(1, int(call_width))
        self.block_size = self.call_width
        self.blocks_per_call = 1

        # Component partition: contiguous block sizes, or arbitrary variant
        # groups gathered into cache order (geno_stream.py:1269-1282).
        self._has_component_partition = (
            component_block_sizes is not None or component_variant_indices is not None
        )
        if component_block_sizes is not None and component_variant_indices is not None:
            raise ValueError(
                "Provide either component_block_sizes or component_variant_indices, not both.")
        if component_variant_indices is not None:
            sizes, cache_to_source = _normalize_component_variant_indices(
                self.source_m, component_variant_indices)
        elif component_block_sizes is not None:
            sizes = _normalize_component_block_sizes(self.source_m, component_block_sizes)
            cache_to_source = np.arange(sum(sizes), dtype=np.int64)
        else:
            sizes = [self.source_m]
            cache_to_source = None
        self._component_block_sizes = sizes
        self._cache_to_source_variant_indices = cache_to_source
        self._has_arbitrary_component_partition = bool(
            cache_to_source is not None
            and not np.array_equal(cache_to_source, np.arange(cache_to_source.size))
        )
        self.m = int(sum(sizes))
        (
            self._block_starts,
            self._block_sizes,
            self._call_component_ids,
            self._component_call_offsets,
        ) = _build_call_geometry(self.m, self.call_width, sizes)
        self._n_calls = int(self._block_starts.size)
        self._n_blocks = self._n_calls
        self._n_components = len(sizes)
        self._call_true_widths = self._block_sizes.copy()
        self._packed_call_widths = ((self._call_true_widths + 3) // 4).astype(np.int32)
        self._call_snp_starts = self._block_starts.astype(np.int32)
        self._max_call_width = int(self._call_true_widths.max())
        self._max_packed_width = int(self._packed_call_widths.max())
        self._max_unpack_width = max(1, 4 * self._max_packed_width)
        self._component_snp_offsets = np.zeros(self._n_components + 1, dtype=np.int32)
        np.cumsum(np.asarray(sizes, dtype=np.int32), out=self._component_snp_offsets[1:])

        self._handle = C.c_void_p()
        self._closed = False
        stream = _lib.stream_ptr()
        synthetic = (
            isinstance(source, SyntheticSource)
            and self._sample_mask is None
            and cache_to_source is None
        )
        from .bed import BedSource

        bed_direct = isinstance(source, BedSource) and cache_to_source is None
        ld_direct = isinstance(source, LDBlockSource) and self._sample_mask is None
        with torch.cuda.device(self.dev):
            if ld_direct:
                # LD-block genotypes generated on the device, permuted into
                # cache order there.
                thr, rho, sfac, quant, _ = source.tables
                sizes_arr = np.asarray(sizes, dtype=np.int32)
                c2s = (None if cache_to_source is None
                       else np.ascontiguousarray(cache_to_source, dtype=np.int64))
                _lib.check(
                    self._lib.coherit_geno_create_ldblock(
                        self.n, self.m, source.block, source.seed, thr.ctypes.data,
                        rho.ctypes.data, sfac.ctypes.data, quant.ctypes.data,
                        None if c2s is None else c2s.ctypes.data, sizes_arr.ctypes.data,
                        len(sizes), self.dev.index, stream, C.byref(self._handle),
                    ),
                    "create LD-block genotypes",
                )
            elif bed_direct:
                # PLINK BED bytes go to the device as they are and are
                # transcoded there (no host repacking).
                sizes_arr = np.asarray(sizes, dtype=np.int32)
                keep = (None if self._sample_mask is None
                        else np.ascontiguousarray(np.flatnonzero(self._sample_mask), dtype=np.int32))
                raw = source.raw_bytes()
                _lib.check(
                    self._lib.coherit_geno_create_bed(
                        raw.ctypes.data, int(raw.size), self._source_n, self.source_m,
                        None if keep is None else keep.ctypes.data,
                        0 if keep is None else int(keep.size), sizes_arr.ctypes.data, len(sizes),
                        self.dev.index, stream, C.byref(self._handle),
                    ),
                    "create genotypes from BED",
                )
            elif synthetic:
                sizes_arr = np.asarray(sizes, dtype=np.int32)
                _lib.check(
                    self._lib.coherit_geno_create_synthetic(
                        self.n, self.m, sizes_arr.ctypes.data, len(sizes), source.seed,
                        source.missing_q24, self.dev.index, stream, C.byref(self._handle),
                    ),
                    "create synthetic genotypes",
                )
            else:
                packed = self._pack_from_source(source)
                _lib.check(
                    self._lib.coherit_geno_create_packed(
                        packed.ctypes.data, self.n, self._n_calls,
                        self._call_true_widths.ctypes.data,
                        self._call_component_ids.ctypes.data, self._n_components, 0,
                        self.dev.index, stream, C.byref(self._handle),
                    ),
                    "create genotypes",
                )
            self._standardization_override = None
            if standardization_override is not None:
                mo, io = standardization_override
                mo = np.ascontiguousarray(mo, dtype=np.float32).reshape(-1)
                io = np.ascontiguousarray(io, dtype=np.float32).reshape(-1)
                if mo.size != self.m or io.size != self.m:
                    raise ValueError(
                        f"standardization_override length mismatch: expected m={self.m}, "
                        f"got means={mo.size}, inv={io.size}."
                    )
                self._standardization_override = (mo, io)
                _lib.check(self._lib.coherit_geno_set_stats(
                    self._handle, 0, None, mo.ctypes.data, io.ctypes.data, stream), "set stats")
            self._refresh_stats()
        self._block_backend_plan = tuple(
            DensePackedBlockDescriptor(
                call_idx=c,
                snp_start=int(self._call_snp_starts[c]),
                true_width=int(self._call_true_widths[c]),
                packed_width=int(self._packed_call_widths[c]),
                storage="hbm_resident_packed",
            )
            for c in range(self._n_calls)
        )
        self._has_sparse_backend = False
        self._exact_diag_dev = None
        # Operator applications issued through this streamer (count, total
        # right-hand-side columns), used to scale per-application costs.
        self.op_stats = {"apps": 0, "cols": 0}

    # ------------------------------------------------------------ building
    def _pack_from_source(self, source) -> np.ndarray:
        lut = _pack_lut(int(source.missing_val))
        parts = []
        cts = self._cache_to_source_variant_indices
        for c in range(self._n_calls):
            s0 = int(self._call_snp_starts[c])
            w = int(self._call_true_widths[c])
            if cts is None:
                blk = source.read_block_variant_major(s0, w)
            else:
                idx = cts[s0:s0 + w]
                lo, hi = int(idx.min()), int(idx.max()) + 1
                blk = source.read_block_variant_major(lo, hi - lo)[idx - lo]
            blk = np.asarray(blk)
            if self._sample_mask is not None:
                blk = blk[:, self._sample_mask]
            parts.append(_pack_block_vm(blk, lut).reshape(-1))
        return np.ascontiguousarray(np.concatenate(parts))

    def _refresh_stats(self) -> None:
        """Read back statistics of slot 0 and build the reference's per-call arrays."""
        m = self.m
        mean = np.zeros(m, dtype=np.float32)
        inv = np.zeros(m, dtype=np.float32)
        cnt = np.zeros(m, dtype=np.int32)
        stream = _lib.stream_ptr()
        if self._standardization_override is None:
            _lib.check(self._lib.coherit_geno_compute_stats(
                self._handle, 0, None, mean.ctypes.data, inv.ctypes.data, cnt.ctypes.data, stream),
                "compute stats")
        else:
            mean, inv = (np.array(x, copy=True) for x in self._standardization_override)
            cnt = None
        G = self._n_components
        ce = np.zeros(G, dtype=np.float64)
        ca = np.zeros(G, dtype=np.float64)
        et = C.c_double()
        at = C.c_double()
        _lib.check(self._lib.coherit_geno_stats_summary(
            self._handle, 0, ce.ctypes.data, ca.ctypes.data, C.byref(et), C.byref(at)), "summary")
        self._means_host = mean if self.keep_host_stats else None
        self._inv_sds_host = inv if self.keep_host_stats else None
        self._count_host = cnt if self.keep_host_stats else None
        self._eff_m_host = float(et.value)
        self._mean_diag_atom_host = float(at.value)
        self._component_eff_m_host = ce.astype(np.float32)
        self._component_mean_diag_atoms_host = ca.astype(np.float32)
        W = self._max_unpack_width
        mbc = np.zeros((self._n_calls, W), dtype=np.float32)
        ibc = np.zeros((self._n_calls, W), dtype=np.float32)
        for c in range(self._n_calls):
            s0 = int(self._call_snp_starts[c])
            tw = int(self._call_true_widths[c])
            mbc[c, :tw] = mean[s0:s0 + tw]
            ibc[c, :tw] = inv[s0:s0 + tw]
        dev = self.dev
        self._means_by_call = torch.as_tensor(mbc, device=dev)
        self._inv_by_call = torch.as_tensor(ibc, device=dev)
        self._eff_m_const = torch.tensor(self._eff_m_host, dtype=torch.float32, device=dev)
        self._component_eff_m_const = torch.as_tensor(self._component_eff_m_host, device=dev)
        self._snp_starts_dev = torch.as_tensor(self._call_snp_starts, device=dev)
        self._true_widths_dev = torch.as_tensor(self._call_true_widths, device=dev)

    # ------------------------------------------------------------ helpers
    def _h(self):
        if self._closed or not self._handle:
            raise RuntimeError("GenoBlockStreamer is closed.")
        return self._handle

    def close(self) -> None:
        if not self._closed and self._handle:
            self._lib.coherit_geno_destroy(self._handle)
        self._closed = True
        self._handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h()

    @property
    def n_components(self) -> int:
        return self._n_components

    @property
    def has_component_partition(self) -> bool:
        return self._has_component_partition

    @property
    def has_arbitrary_component_partition(self) -> bool:
        return self._has_arbitrary_component_partition

    @property
    def has_sparse_backend(self) -> bool:
        return False

    def block_backend_plan(self):
        return self._block_backend_plan

    def component_source_variant_indices(self, component_idx: int) -> np.ndarray:
        if not self._has_component_partition or self._cache_to_source_variant_indices is None:
            raise ValueError("Component source SNP indices require component-partitioned streamer geometry.")
        if component_idx < 0 or component_idx >= self._n_components:
            raise IndexError(
                f"component_idx={component_idx} out of range for {self._n_components} components."
            )
        s0 = int(self._component_snp_offsets[component_idx])
        s1 = int(self._component_snp_offsets[component_idx + 1])
        return np.asarray(self._cache_to_source_variant_indices[s0:s1], dtype=np.int64)

    def info(self) -> dict:
        vals = [C.c_int64() for _ in range(4)]
        g = C.c_int32()
        miss = C.c_int64()
        dbytes = C.c_int64()
        _lib.check(self._lib.coherit_geno_info(
            self._h(), *(C.byref(v) for v in vals), C.byref(g), C.byref(miss), C.byref(dbytes)))
        return dict(n=vals[0].value, m=vals[1].value, n_pad=vals[2].value, m_pad=vals[3].value,
                    n_components=g.value, n_missing=miss.value, device_bytes=dbytes.value)

    def reserve(self, k_max: int, precision: str | None = None) -> None:
        """Pre-size the operator workspace (no allocation in later calls)."""
        prec = _lib.PRECISIONS[precision or self.precision]
        _lib.check(self._lib.coherit_geno_reserve(self._h(), int(k_max), prec), "reserve")

    def autotune(self, widths, precision: str | None = None, reps: int = 2) -> list:
        """Time candidate launch configurations of the operator for each
        width (stage size, ring depths, split-K grid, row tiles per CTA, CTAs
        per cluster sharing each B tile) on these genotypes and
        keep the fastest for later launches of that width and precision
        (coherit_geno_autotune).  Returns one record per width."""
        out = []
        prec = self._prec_code(precision)
        for k in widths:
            ch = (C.c_int32 * 8)()
            best, dflt = C.c_float(), C.c_float()
            _lib.check(self._lib.coherit_geno_autotune(
                self._h(), int(k), prec, int(reps), ch, C.byref(best), C.byref(dflt),
                _lib.stream_ptr()), "autotune")
            out.append({"k": int(k), "precision": precision or self.precision,
                        "four_block_stages": bool(ch[0]), "a_ring": int(ch[1]),
                        "b_ring": int(ch[2]), "g_ring": int(ch[6]), "grid_x_sms": int(ch[3]),
                        "cluster": int(ch[5]), "tiles_per_cta": int(ch[7]),
                        "candidates": int(ch[4]),
                        "best_ms": round(best.value, 4), "default_ms": round(dflt.value, 4)})
        return out

    def set_launch(self, k: int, precision: str | None = None, *, four_block_stages: bool = True,
                   a_ring: int = 0, b_ring: int = 0, grid_x_sms: int = 4, cluster: int = 1,
                   g_ring: int = 0, tiles: int = 1, policy: bool = False) -> None:
        """Pin the launch configuration of width k (coherit_geno_set_launch);
        ``policy=True`` returns the width to the fixed policy."""
        prec = self._prec_code(precision)
        if policy:
            _lib.check(self._lib.coherit_geno_set_launch(self._h(), int(k), prec, None),
                       "set_launch")
            return
        cfg = (C.c_int32 * 8)(int(bool(four_block_stages)), int(a_ring), int(b_ring),
                              int(grid_x_sms), 0, int(cluster), int(g_ring), int(tiles))
        _lib.check(self._lib.coherit_geno_set_launch(self._h(), int(k), prec, cfg), "set_launch")

    def _prec_code(self, precision) -> int:
        return self._prec if precision is None else _lib.PRECISIONS[precision]

    def _kv_raw(self, V, *, comp_scale, mode=_lib.MODE_SUM, theta_e=None, snp_weight=None,
                slot=0, precision=None):
        V, squeeze = as_rhs(V, self.dev)
        if V.shape[0] != self.n:
            raise ValueError(f"V has {V.shape[0]} rows, expected n={self.n}")
        k = int(V.shape[1])
        G = self._n_components
        if mode == _lib.MODE_STACKED:
            out = torch.empty((G, self.n, k), dtype=torch.float32, device=self.dev)
        else:
            out = torch.empty((self.n, k), dtype=torch.float32, device=self.dev)
        if k == 0:
            return out
        self.op_stats["apps"] += 1
        self.op_stats["cols"] += k
        cs = np.ascontiguousarray(comp_scale, dtype=np.float32)
        if cs.size != G:
            raise ValueError(f"expected {G} component scales, got {cs.size}")
        sw = None
        if snp_weight is not None:
            sw = torch.as_tensor(snp_weight, dtype=torch.float32, device=self.dev).contiguous()
            if sw.numel() != self.m:
                raise ValueError("snp_weight must have one entry per SNP")
        _lib.check(self._lib.coherit_geno_kv(
            self._h(), int(slot), int(mode), self._prec_code(precision), V.data_ptr(), k, k,
            cs.ctypes.data, 0 if theta_e is None else 1, 0.0 if theta_e is None else float(theta_e),
            _lib.ptr(sw), out.data_ptr(), k, _lib.stream_ptr()), "kv")
        if squeeze:
            return out[..., 0]
        return out

    def _inv_eff(self, eff: float) -> float:
        return 1.0 / eff if eff > 0 else 1.0

    # ------------------------------------------------------------ operators
    def kv(self, V, normalize: bool = True, *, precision=None):
        """K V = Z Z^T V / m_eff over all SNPs (geno_stream.py:2669-2679)."""
        s = self._inv_eff(self._eff_m_host) if normalize else 1.0
        return self._kv_raw(V, comp_scale=np.full(self._n_components, s), precision=precision)

    def component_kv(self, V, component_idx: int, normalize: bool = True, *, precision=None):
        if component_idx < 0 or component_idx >= self._n_components:
            raise IndexError(
                f"component_idx={component_idx} out of range for {self._n_components} components."
            )
        scale = np.zeros(self._n_components)
        eff = float(self._component_eff_m_host[component_idx])
        scale[component_idx] = self._inv_eff(eff) if normalize else 1.0
        if self._n_components == 1:
            return self._kv_raw(V, comp_scale=scale, precision=precision)
        return self._kv_raw(V, comp_scale=scale, mode=_lib.MODE_STACKED,
                            precision=precision)[component_idx]

    def stacked_component_kv(self, V, normalize: bool = True, *, precision=None):
        scale = np.asarray([
            self._inv_eff(float(e)) if normalize else 1.0 for e in self._component_eff_m_host
        ])
        return self._kv_raw(V, comp_scale=scale, mode=_lib.MODE_STACKED, precision=precision)

    def weighted_component_hv(self, theta_g, theta_e, V, *, precision=None):
        """sum_g theta_g K_g V (+ theta_e V) in one genome pass (kv_impl.py:1089-1135)."""
        tg = np.asarray(theta_g.detach().cpu() if isinstance(theta_g, torch.Tensor) else theta_g,
                        dtype=np.float64).reshape(-1)
        if tg.size != self._n_components:
            raise ValueError(
                f"theta_g length mismatch: expected {self._n_components}, got {tg.size}."
            )
        eff = self._component_eff_m_host.astype(np.float64)
        scale = np.where(eff > 0, tg / np.where(eff > 0, eff, 1.0), 0.0)
        te = None
        if theta_e is not None:
            te = float(theta_e.detach().cpu().reshape(-1)[0]) if isinstance(theta_e, torch.Tensor) \
                else float(np.asarray(theta_e).reshape(-1)[0])
        return self._kv_raw(V, comp_scale=scale, theta_e=te, precision=precision)

    def snp_weighted_kv(self, V, weights, denom, *, precision=None):
        """Z diag(w) Z^T V / denom (kv_impl.py:329-379)."""
        d = float(denom)
        return self._kv_raw(V, comp_scale=np.full(self._n_components, 1.0 / d),
                            snp_weight=weights, precision=precision)

    def xtv(self, V, normalize: bool = False, *, precision=None):
        """X^T V = inv_sd * diff^T V (m x k) (geno_stream.py:2736-2747)."""
        V, squeeze = as_rhs(V, self.dev)
        if V.shape[0] != self.n:
            raise ValueError(f"V has {V.shape[0]} rows, expected n={self.n}")
        k = int(V.shape[1])
        out = torch.empty((self.m, k), dtype=torch.float32, device=self.dev)
        s = self._inv_eff(self._eff_m_host) if normalize else 1.0
        cs = np.full(self._n_components, s, dtype=np.float32)
        _lib.check(self._lib.coherit_geno_xtv(
            self._h(), 0, self._prec_code(precision), V.data_ptr(), k, k, cs.ctypes.data,
            out.data_ptr(), k, _lib.stream_ptr()), "xtv")
        return out[:, 0] if squeeze else out

    def zxb(self, b, *, precision=None):
        """Z b = sum_j diff_ij inv_sd_j b_j for b of shape (m,) or (m, C)."""
        b = torch.as_tensor(b, dtype=torch.float32, device=self.dev)
        squeeze = b.ndim == 1
        if squeeze:
            b = b[:, None]
        b = b.contiguous()
        if b.shape[0] != self.m:
            raise ValueError(f"b has {b.shape[0]} rows, expected m={self.m}")
        Cc = int(b.shape[1])
        out = torch.empty((self.n, Cc), dtype=torch.float32, device=self.dev)
        _lib.check(self._lib.coherit_geno_zxb(
            self._h(), 0, self._prec_code(precision), b.data_ptr(), Cc, Cc, out.data_ptr(), Cc,
            _lib.stream_ptr()), "zxb")
        return out[:, 0] if squeeze else out

    def diag(self) -> torch.Tensor:
        """Exact mean diagonal atom tr(K)/n (geno_stream.py:2773-2778)."""
        return torch.tensor(self._mean_diag_atom_host, dtype=torch.float32, device=self.dev)

    def component_diag_list(self) -> list:
        return [torch.tensor(float(a), dtype=torch.float32, device=self.dev)
                for a in self._component_mean_diag_atoms_host]

    def set_standardization(self, means, inv_sds) -> None:
        """Install externally supplied per-SNP means and inverse sds (cache
        order), e.g. the training set's on a test streamer before prediction
        (reml_model.py:275-279)."""
        mo = np.ascontiguousarray(means, dtype=np.float32).reshape(-1)
        io = np.ascontiguousarray(inv_sds, dtype=np.float32).reshape(-1)
        if mo.size != self.m or io.size != self.m:
            raise ValueError(f"standardization length mismatch: expected m={self.m}, "
                             f"got means={mo.size}, inv={io.size}.")
        self._standardization_override = (mo, io)
        with torch.cuda.device(self.dev):
            _lib.check(self._lib.coherit_geno_set_stats(
                self._h(), 0, None, mo.ctypes.data, io.ctypes.data, _lib.stream_ptr()), "set stats")
            self._refresh_stats()

    def standardized_columns(self, snp_indices) -> torch.Tensor:
        """Device FP32 (n, len(snp_indices)) standardised genotype columns
        (cache SNP order; missing -> 0), computed from the resident matrix."""
        idx = np.asarray(snp_indices, dtype=np.int64)
        if idx.ndim != 1:
            raise ValueError("snp_indices must be 1D.")
        if idx.size and (idx.min() < 0 or idx.max() >= self.m):
            raise IndexError("snp_indices out of range.")
        out = torch.empty((self.n, idx.size), dtype=torch.float32, device=self.dev)
        if idx.size == 0:
            return out
        idx_dev = torch.as_tensor(idx, device=self.dev)
        _lib.check(self._lib.coherit_geno_extract_columns(
            self._h(), 0, idx_dev.data_ptr(), int(idx.size), out.data_ptr(), int(idx.size),
            _lib.stream_ptr()), "extract columns")
        return out

    def extract_standardized_columns(self, snp_indices: np.ndarray) -> np.ndarray:
        """Host FP32 (n, len(snp_indices)) standardised columns
        (geno_stream.py:2748-2760)."""
        return self.standardized_columns(snp_indices).cpu().numpy()

    def exact_diag(self, *, target_block_bytes: int = 256 * 1024 * 1024) -> torch.Tensor:
        """Sample-wise diagonal of the GRM, cached (geno_stream.py:2780-2821)."""
        if self._exact_diag_dev is not None:
            return self._exact_diag_dev
        out = torch.empty(self.n, dtype=torch.float32, device=self.dev)
        _lib.check(self._lib.coherit_geno_exact_diag(self._h(), 0, out.data_ptr(),
                                                     _lib.stream_ptr()), "exact_diag")
        self._exact_diag_dev = out
        return out

    def build_projected_core_atom(self, U, *, subtract_identity: bool = True):
        """U^T K U (- I) for the whole matrix (kv_impl.py:1190-1229)."""
        XtU = self.xtv(U)
        core = XtU.T @ XtU
        eff = self._eff_m_host
        if eff <= 0:
            return torch.zeros_like(core)
        core = core / eff
        if subtract_identity:
            core = core - torch.eye(core.shape[0], device=core.device, dtype=core.dtype)
        return core

    def build_projected_core_atoms(self, U, *, subtract_identity: bool = True):
        """Per-component U^T K_g U (- I) (kv_impl.py:1287-1339)."""
        if not self._has_component_partition:
            raise ValueError("Projected-core atoms require component-partitioned streamer geometry.")
        XtU = self.xtv(U)
        cores = []
        for g in range(self._n_components):
            s0 = int(self._component_snp_offsets[g])
            s1 = int(self._component_snp_offsets[g + 1])
            blk = XtU[s0:s1]
            core = blk.T @ blk
            eff = float(self._component_eff_m_host[g])
            if eff > 0:
                core = core / eff
                if subtract_identity:
                    core = core - torch.eye(core.shape[0], device=core.device, dtype=core.dtype)
            else:
                core = torch.zeros_like(core)
            cores.append(core)
        return torch.stack(cores)

    # ---------------------------------------------------- reference access
    def _pop_cached(self, call_idx) -> np.ndarray:
        """Reference-layout packed block of call `call_idx` (n, ceil(w/4)) uint8."""
        c = int(call_idx)
        w = int(self._call_true_widths[c])
        out = np.empty((self.n, (w + 3) // 4), dtype=np.uint8)
        _lib.check(self._lib.coherit_geno_read_packed(
            self._h(), int(self._call_snp_starts[c]), w, out.ctypes.data, _lib.stream_ptr()),
            "read packed")
        return out

    _packed_block_host = _pop_cached

    def _prepare_kv_pass(self) -> None:
        self._h()

    def check(self) -> None:
        """Raise if a kernel of this handle gave up on a bounded device wait."""
        _lib.check(self._lib.coherit_geno_check(self._h(), _lib.stream_ptr()), "device check")


class BedBlockStreamer(GenoBlockStreamer):
    """``BedBlockStreamer(bed_prefix, ...)`` alias (geno_stream.py:2867-2896)."""

    def __init__(self, bed_prefix: str, call_width: int = 131072, component_block_sizes=None,
                 component_variant_indices=None, standardization_override=None, device=None,
                 keep_host_stats: bool = True, build_threads: int | None = None,
                 sample_mask: np.ndarray | None = None, ring_depth: int | None = None,
                 source_build_chunk_width: int | None = None, *, precision: str | None = None):
        super().__init__(bed_prefix=bed_prefix, call_width=call_width,
                         component_block_sizes=component_block_sizes,
                         component_variant_indices=component_variant_indices,
                         standardization_override=standardization_override, device=device,
                         keep_host_stats=keep_host_stats, build_threads=build_threads,
                         sample_mask=sample_mask, ring_depth=ring_depth,
                         source_build_chunk_width=source_build_chunk_width, precision=precision)


__all__ = [
    "ArraySource",
    "SyntheticSource",
    "GenoBlockStreamer",
    "BedBlockStreamer",
    "as_rhs",
]
