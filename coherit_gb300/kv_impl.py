"""Streaming-driver entry points with the signatures of GPU_REML's kv_impl.py.

The reference drives one jitted kernel per call block and streams each
packed block from the host (kv_impl.py:268-1339).  Here the genotypes are
resident in HBM; when ``pop_block`` / ``streamers`` are this package's
``GenoBlockStreamer`` objects the functions dispatch straight to the
resident operator (one or two kernel launches per application).  Any other
``pop_block`` callable is honoured too: its blocks and the given per-call
statistics are uploaded once into a transient resident matrix, so callers
that build blocks themselves keep working.

Mathematical contract (kv_impl.py:9-12):
    out = (1/eff_m) * sum_c Z_c (Z_c^T V)
with Z_c the mean-imputed, centred, 1/sd-scaled genotypes of call c.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Sequence

import numpy as np
import torch

from . import _lib
from .geno_stream import GenoBlockStreamer, as_rhs


def _owner(pop_block) -> GenoBlockStreamer | None:
    owner = getattr(pop_block, "__self__", None)
    return owner if isinstance(owner, GenoBlockStreamer) else None


def _flat_stats(true_widths, means_by_call, inv_by_call):
    tw = np.asarray(torch.as_tensor(true_widths).cpu(), dtype=np.int64).reshape(-1)
    mb = np.asarray(torch.as_tensor(means_by_call).cpu(), dtype=np.float32)
    ib = np.asarray(torch.as_tensor(inv_by_call).cpu(), dtype=np.float32)
    mean = np.concatenate([mb[c, : tw[c]] for c in range(tw.size)]) if tw.size else np.zeros(0, np.float32)
    inv = np.concatenate([ib[c, : tw[c]] for c in range(tw.size)]) if tw.size else np.zeros(0, np.float32)
    return tw, np.ascontiguousarray(mean), np.ascontiguousarray(inv)


class _TransientGeno:
    """Resident copy of caller-supplied packed blocks with given statistics."""

    def __init__(self, n, n_calls, pop_block, true_widths, means_by_call, inv_by_call, device):
        self.lib = _lib.load()
        tw, mean, inv = _flat_stats(true_widths, means_by_call, inv_by_call)
        blocks = []
        for c in range(n_calls):
            blk = np.ascontiguousarray(np.asarray(pop_block(c), dtype=np.uint8))
            pw = (int(tw[c]) + 3) // 4
            if blk.shape != (n, pw):
                raise ValueError(f"pop_block({c}) returned {blk.shape}, expected {(n, pw)}")
            blocks.append(blk.reshape(-1))
        packed = np.ascontiguousarray(np.concatenate(blocks))
        widths = tw.astype(np.int32)
        self.h = C.c_void_p()
        self.n = n
        self.m = int(tw.sum())
        self.dev = device
        stream = _lib.stream_ptr()
        _lib.check(self.lib.coherit_geno_create_packed(
            packed.ctypes.data, n, n_calls, widths.ctypes.data, None, 1, 0, device.index, stream,
            C.byref(self.h)), "transient genotypes")
        _lib.check(self.lib.coherit_geno_set_stats(
            self.h, 0, None, mean.ctypes.data, inv.ctypes.data, stream), "transient stats")

    def kv(self, V, scale, snp_weight=None, precision=_lib.PREC_BF16X3):
        V2, squeeze = as_rhs(V, self.dev)
        k = V2.shape[1]
        out = torch.empty_like(V2)
        cs = np.asarray([scale], np.float32)
        sw = None if snp_weight is None else torch.as_tensor(snp_weight, dtype=torch.float32,
                                                            device=self.dev).contiguous()
        _lib.check(self.lib.coherit_geno_kv(
            self.h, 0, _lib.MODE_SUM, precision, V2.data_ptr(), k, k, cs.ctypes.data, 0, 0.0,
            _lib.ptr(sw), out.data_ptr(), k, _lib.stream_ptr()), "kv")
        return out[:, 0] if squeeze else out

    def xtv(self, V, scale, precision=_lib.PREC_BF16X3):
        V2, squeeze = as_rhs(V, self.dev)
        k = V2.shape[1]
        out = torch.empty((self.m, k), dtype=torch.float32, device=self.dev)
        cs = np.asarray([scale], np.float32)
        _lib.check(self.lib.coherit_geno_xtv(
            self.h, 0, precision, V2.data_ptr(), k, k, cs.ctypes.data, out.data_ptr(), k,
            _lib.stream_ptr()), "xtv")
        return out[:, 0] if squeeze else out

    def zxb(self, b, precision=_lib.PREC_BF16X3):
        b = torch.as_tensor(b, dtype=torch.float32, device=self.dev)
        squeeze = b.ndim == 1
        b2 = (b[:, None] if squeeze else b).contiguous()
        Cc = b2.shape[1]
        out = torch.empty((self.n, Cc), dtype=torch.float32, device=self.dev)
        _lib.check(self.lib.coherit_geno_zxb(
            self.h, 0, precision, b2.data_ptr(), Cc, Cc, out.data_ptr(), Cc, _lib.stream_ptr()),
            "zxb")
        return out[:, 0] if squeeze else out

    def close(self):
        if self.h:
            self.lib.coherit_geno_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _device(V) -> torch.device:
    if isinstance(V, torch.Tensor) and V.is_cuda:
        return V.device
    return torch.device("cuda", torch.cuda.current_device())


def _zero_rhs(V) -> torch.Tensor:
    """Zero result of V's shape on V's device (no call blocks to apply)."""
    V2 = V if isinstance(V, torch.Tensor) else torch.as_tensor(np.asarray(V, dtype=np.float32))
    if V2.ndim not in (1, 2):
        raise ValueError(f"right-hand side must be 1-D or 2-D, got shape {tuple(V2.shape)}")
    return torch.zeros(V2.shape, dtype=torch.float32, device=V2.device)


def _eff(eff_m) -> float:
    return float(torch.as_tensor(eff_m).reshape(()).item())


def kv_impl_streamed(V, true_widths, means_by_call, inv_by_call, eff_m, *, n: int, n_calls: int,
                     pop_block: Callable[[int], np.ndarray], missing_val: int = 3,
                     normalize: bool = True):
    """K V over all call blocks (kv_impl.py:268-326)."""
    if int(missing_val) != 3:
        raise ValueError("packed genotypes use code 3 for missing values")
    eff = _eff(eff_m)
    scale = (1.0 / eff) if (normalize and eff > 0) else 1.0
    st = _owner(pop_block)
    if st is not None and means_by_call is st._means_by_call and inv_by_call is st._inv_by_call:
        return st._kv_raw(V, comp_scale=np.full(st.n_components, scale))
    if n_calls == 0:
        return _zero_rhs(V)
    tg = _TransientGeno(n, n_calls, pop_block, true_widths, means_by_call, inv_by_call, _device(V))
    try:
        return tg.kv(V, scale)
    finally:
        tg.close()


def kv_impl_snp_weighted_streamed(V, true_widths, means_by_call, inv_by_call, weights_by_call,
                                  denom, *, n: int, n_calls: int, pop_block, missing_val: int = 3):
    """Z diag(w) Z^T V / denom for per-SNP weights (kv_impl.py:329-379)."""
    if int(missing_val) != 3:
        raise ValueError("packed genotypes use code 3 for missing values")
    if n_calls == 0:
        # No call blocks: the accumulator stays zero (kv_impl.py:358-359).
        return _zero_rhs(V)
    tw, _, _ = _flat_stats(true_widths, means_by_call, inv_by_call)
    wb = np.asarray(torch.as_tensor(weights_by_call).cpu(), dtype=np.float32)
    w = np.concatenate([wb[c, : tw[c]] for c in range(tw.size)]) if tw.size else np.zeros(0, np.float32)
    d = float(torch.as_tensor(denom).reshape(()).item())
    st = _owner(pop_block)
    if st is not None and means_by_call is st._means_by_call and inv_by_call is st._inv_by_call:
        return st.snp_weighted_kv(V, w, d)
    tg = _TransientGeno(n, n_calls, pop_block, true_widths, means_by_call, inv_by_call, _device(V))
    try:
        return tg.kv(V, 1.0 / d, snp_weight=w)
    finally:
        tg.close()


def xtv_impl_streamed(V, m: int, snp_starts, true_widths, means_by_call, inv_by_call, *,
                      n_calls: int, pop_block, missing_val: int = 3, normalize: bool = False,
                      eff_m=None):
    """X^T V = inv_sd * diff^T V, shape (m, k) (kv_impl.py:382-439)."""
    if normalize and eff_m is None:
        raise ValueError("xtv_impl_streamed(normalize=True) requires eff_m.")
    scale = 1.0
    if normalize:
        eff = _eff(eff_m)
        scale = 1.0 / eff if eff > 0 else 1.0
    st = _owner(pop_block)
    if st is not None and means_by_call is st._means_by_call and inv_by_call is st._inv_by_call:
        out = st.xtv(V, normalize=False)
        return out * scale if scale != 1.0 else out
    n = as_rhs(V, _device(V))[0].shape[0]
    tg = _TransientGeno(n, n_calls, pop_block, true_widths, means_by_call, inv_by_call, _device(V))
    try:
        return tg.xtv(V, scale)
    finally:
        tg.close()


def xtv_impl_multi_streamed(V, streamers: Sequence[GenoBlockStreamer], call_plan, *,
                            missing_val: int = 3, normalize: bool = False):
    """Per-streamer X^T V (kv_impl.py:442-497)."""
    if not streamers:
        raise ValueError("xtv_impl_multi_streamed requires at least one streamer.")
    return tuple(st.xtv(V, normalize=normalize) for st in streamers)


def xtv_impl_multi_streamed_concat(V, streamers, call_plan, *, missing_val: int = 3,
                                   normalize: bool = False):
    parts = xtv_impl_multi_streamed(V, streamers, call_plan, missing_val=missing_val,
                                    normalize=normalize)
    return parts[0] if len(parts) == 1 else torch.cat(parts, dim=0)


def zxb_impl_streamed(b_by_call, true_widths, means_by_call, inv_by_call, *, n: int, n_calls: int,
                      pop_block, missing_val: int = 3, component_ids=None, n_components: int = 0):
    """Test prediction g = Z b, total and per component (kv_impl.py:524-602)."""
    bb = torch.as_tensor(b_by_call)
    if bb.ndim != 2:
        raise ValueError("zxb_impl_streamed expects b_by_call with shape (n_calls, max_unpack_width).")
    if bb.shape[0] != int(n_calls):
        raise ValueError(
            f"zxb_impl_streamed b_by_call row mismatch: expected n_calls={int(n_calls)}, "
            f"got {int(bb.shape[0])}.")
    tws, mbs, ibs = (tuple(torch.as_tensor(x).shape)
                     for x in (true_widths, means_by_call, inv_by_call))
    if len(tws) != 1 or tws[0] != int(n_calls):
        raise ValueError(f"zxb_impl_streamed true_widths must have shape ({int(n_calls)},), "
                         f"got {tws}.")
    if len(mbs) != 2 or mbs[0] != int(n_calls):
        raise ValueError("zxb_impl_streamed means_by_call must have shape "
                         f"(n_calls, max_unpack_width), got {mbs}.")
    if ibs != mbs:
        raise ValueError(f"zxb_impl_streamed inv_by_call shape mismatch: expected {mbs}, "
                         f"got {ibs}.")
    tw, _, _ = _flat_stats(true_widths, means_by_call, inv_by_call)
    if component_ids is not None:
        component_ids = np.asarray(component_ids, dtype=np.int32).reshape(-1)
        if component_ids.shape[0] != int(n_calls):
            raise ValueError(
                f"zxb_impl_streamed component_ids must have shape ({int(n_calls)},), "
                f"got {component_ids.shape}.")
        if int(n_components) <= 0:
            raise ValueError("zxb_impl_streamed requires n_components > 0 when component_ids is provided.")
        if np.any(component_ids < 0) or np.any(component_ids >= int(n_components)):
            raise ValueError(
                f"zxb_impl_streamed component_ids entries must lie in [0, {int(n_components)}).")
    dev = bb.device if bb.is_cuda else torch.device("cuda", torch.cuda.current_device())
    bbc = bb.to(dev, torch.float32)
    flat = torch.cat([bbc[c, : int(tw[c])] for c in range(int(n_calls))]) if n_calls else \
        torch.zeros(0, device=dev)
    st = _owner(pop_block)
    runner = st if (st is not None and means_by_call is st._means_by_call
                    and inv_by_call is st._inv_by_call) else None
    tg = None
    if runner is None:
        tg = _TransientGeno(n, n_calls, pop_block, true_widths, means_by_call, inv_by_call, dev)
        runner = tg
    try:
        if component_ids is None:
            total = runner.zxb(flat)
            return total, tuple(torch.zeros(n, device=dev) for _ in range(int(n_components)))
        starts = np.concatenate([[0], np.cumsum(tw)])
        B = torch.zeros((flat.shape[0], int(n_components)), device=dev)
        for c in range(int(n_calls)):
            B[starts[c]: starts[c + 1], int(component_ids[c])] = flat[starts[c]: starts[c + 1]]
        comps = runner.zxb(B)
        return comps.sum(dim=1), tuple(comps[:, g] for g in range(int(n_components)))
    finally:
        if tg is not None:
            tg.close()


def _stack_b_by_call(b_by_call_stack: torch.Tensor, true_widths, calls=None) -> torch.Tensor:
    """(C, n_calls, width) per-call effect rows -> (sum of true widths, C) in
    cache SNP order; calls outside ``calls`` (when given) contribute zeros."""
    tw = np.asarray(torch.as_tensor(true_widths).cpu(), dtype=np.int64).reshape(-1)
    starts = np.concatenate([[0], np.cumsum(tw)])
    C = int(b_by_call_stack.shape[0])
    B = torch.zeros((int(starts[-1]), C), dtype=torch.float32, device=b_by_call_stack.device)
    for c in (range(tw.size) if calls is None else sorted(set(int(x) for x in calls))):
        w = int(tw[c])
        B[starts[c]: starts[c] + w] = b_by_call_stack[:, c, :w].T.to(torch.float32)
    return B


def zxb_impl_same_stream_multi(b_by_call_stack, true_widths, means_by_call, inv_by_call, *,
                               n: int, n_calls: int, pop_block, missing_val: int = 3):
    """Several components' predictions over one genotype matrix (kv_impl.py:605-661):
    the C effect vectors become the C columns of one Z B launch."""
    bs = torch.as_tensor(b_by_call_stack)
    if bs.ndim != 3:
        raise ValueError("zxb_impl_same_stream_multi expects shape "
                         "(n_components, n_calls, max_unpack_width).")
    n_components = int(bs.shape[0])
    if n_components <= 0:
        raise ValueError("zxb_impl_same_stream_multi requires at least one component.")
    if int(bs.shape[1]) != int(n_calls):
        raise ValueError(f"zxb_impl_same_stream_multi call mismatch: expected {int(n_calls)}, "
                         f"got {int(bs.shape[1])}.")
    if int(missing_val) != 3:
        raise ValueError("packed genotypes use code 3 for missing values")
    dev = bs.device if bs.is_cuda else torch.device("cuda", torch.cuda.current_device())
    if int(n_calls) == 0:
        zero = torch.zeros((int(n), n_components), device=dev)
        return zero.sum(dim=1), tuple(zero[:, i] for i in range(n_components))
    B = _stack_b_by_call(bs.to(dev), true_widths)
    st = _owner(pop_block)
    runner = st if (st is not None and means_by_call is st._means_by_call
                    and inv_by_call is st._inv_by_call) else None
    tg = None
    if runner is None:
        tg = _TransientGeno(n, n_calls, pop_block, true_widths, means_by_call, inv_by_call, dev)
        runner = tg
    try:
        comps = runner.zxb(B)
        return comps.sum(dim=1), tuple(comps[:, i] for i in range(n_components))
    finally:
        if tg is not None:
            tg.close()


def zxb_impl_multi_streamed(b_by_call_list, streamers: Sequence[GenoBlockStreamer], call_plan, *,
                            missing_val: int = 3):
    """Multi-GRM test prediction: sum over streamers of Z_g b_g, over the calls
    ``call_plan`` lists, and each term (kv_impl.py:664-724)."""
    if len(b_by_call_list) != len(streamers):
        raise ValueError(f"zxb_impl_multi_streamed b_by_call_list length mismatch: "
                         f"expected {len(streamers)}, got {len(b_by_call_list)}.")
    if not streamers:
        raise ValueError("zxb_impl_multi_streamed requires at least one streamer.")
    if int(missing_val) != 3:
        raise ValueError("packed genotypes use code 3 for missing values")
    bl = [torch.as_tensor(b) for b in b_by_call_list]
    for g, (b, st) in enumerate(zip(bl, streamers)):
        if b.ndim != 2:
            raise ValueError(f"zxb_impl_multi_streamed expects b_by_call_list[{g}] to be 2D, "
                             f"got ndim={b.ndim}.")
        if int(b.shape[0]) != int(st._n_calls):
            raise ValueError(f"zxb_impl_multi_streamed row mismatch for component {g}: "
                             f"expected n_calls={int(st._n_calls)}, got {int(b.shape[0])}.")
    dev = streamers[0].dev
    n = int(streamers[0].n)
    comps = [torch.zeros(n, device=dev) for _ in streamers]
    calls_of = [[] for _ in streamers]
    for g, c in call_plan:
        calls_of[int(g)].append(int(c))
    for g, st in enumerate(streamers):
        if calls_of[g]:
            B = _stack_b_by_call(bl[g].to(dev)[None], st._call_true_widths, calls_of[g])
            comps[g] = st.zxb(B[:, 0])
    total = torch.zeros(n, device=dev)
    for c in comps:
        total = total + c
    return total, tuple(comps)


def kv_impl_multi_streamed_weighted(V, streamers: Sequence[GenoBlockStreamer], call_plan, theta_g,
                                    *, theta_e=None, missing_val: int = 3):
    """sum_g theta_g K_g V (+ theta_e V) over several streamers (kv_impl.py:911-973)."""
    if not streamers:
        raise ValueError("kv_impl_multi_streamed_weighted requires at least one streamer.")
    tg = np.asarray(torch.as_tensor(theta_g).cpu(), dtype=np.float64).reshape(-1)
    acc = None
    for g, st in enumerate(streamers):
        term = st.weighted_component_hv(np.full(st.n_components, tg[g]),
                                        theta_e if (g == 0 and theta_e is not None) else None, V)
        acc = term if acc is None else acc + term
    return acc


def kv_impl_multi_streamed_stacked(V, streamers, call_plan, *, missing_val: int = 3,
                                  normalize: bool = True):
    """One K_g V per streamer stacked on axis 0 (kv_impl.py:976-1039)."""
    if not streamers:
        raise ValueError("kv_impl_multi_streamed_stacked requires at least one streamer.")
    return torch.stack([st.kv(V, normalize=normalize) for st in streamers])


def kv_impl_partitioned_component(V, streamer: GenoBlockStreamer, *, component_idx: int,
                                  missing_val: int = 3, normalize: bool = True):
    """kv_impl.py:1042-1086"""
    return streamer.component_kv(V, component_idx, normalize=normalize)


def kv_impl_partitioned_weighted(V, streamer: GenoBlockStreamer, theta_g, *, theta_e=None,
                                 missing_val: int = 3):
    """kv_impl.py:1089-1135"""
    return streamer.weighted_component_hv(theta_g, theta_e, V)


def kv_impl_partitioned_stacked(V, streamer: GenoBlockStreamer, *, missing_val: int = 3,
                                normalize: bool = True):
    """kv_impl.py:1138-1187"""
    return streamer.stacked_component_kv(V, normalize=normalize)


def build_projected_core_atom_streamed(U, streamer: GenoBlockStreamer, *, missing_val: int = 3,
                                       subtract_identity: bool = True):
    """kv_impl.py:1190-1229"""
    if torch.as_tensor(U).ndim != 2:
        raise ValueError("build_projected_core_atom_streamed expects U with shape (n, k).")
    return streamer.build_projected_core_atom(U, subtract_identity=subtract_identity)


def build_projected_core_atoms_multi_streamed(U, streamers, call_plan, *, missing_val: int = 3,
                                              subtract_identity: bool = True):
    """kv_impl.py:1232-1285"""
    if torch.as_tensor(U).ndim != 2:
        raise ValueError("build_projected_core_atoms_multi_streamed expects U with shape (n, k).")
    if not streamers:
        raise ValueError("build_projected_core_atoms_multi_streamed requires at least one streamer.")
    return torch.stack([st.build_projected_core_atom(U, subtract_identity=subtract_identity)
                        for st in streamers])


def build_projected_core_atoms_partitioned(U, streamer: GenoBlockStreamer, *, missing_val: int = 3,
                                           subtract_identity: bool = True):
    """kv_impl.py:1287-1339"""
    if torch.as_tensor(U).ndim != 2:
        raise ValueError("build_projected_core_atoms_partitioned expects U with shape (n, k).")
    return streamer.build_projected_core_atoms(U, subtract_identity=subtract_identity)


# ------------------------------------------------------ rare-variant shards

def _host(x) -> np.ndarray:
    """Host numpy view of a numpy array or (device) tensor."""
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


class _TransientSparse:
    """A resident sparse matrix built from one shard's host entry arrays
    (csc_all_rows / cols / vals, columns local to the shard and ascending,
    sparse_stream.py:1037-1145) with the shard's own statistics installed."""

    def __init__(self, n, m, mean, inv, rows, cols, vals, device):
        self._lib = _lib.load()
        self.n, self.m = int(n), int(m)
        rows = np.ascontiguousarray(_host(rows), dtype=np.int32).reshape(-1)
        cols = _host(cols).astype(np.int64, copy=False).reshape(-1)
        vals = _host(vals).reshape(-1)
        if not (rows.size == cols.size == vals.size):
            raise ValueError("csc_all_rows, csc_all_cols and csc_all_vals must have one length.")
        if cols.size and (np.any(np.diff(cols) < 0) or cols[0] < 0 or cols[-1] >= self.m):
            raise ValueError("csc_all_cols must be ascending shard-local SNP indices in [0, m).")
        if vals.dtype == np.int8:
            codes = vals
        else:
            # Merged float values are 1 (het), 2 (hom-alt) or the SNP mean
            # (missing, sparse_stream.py:609-647); a missing entry whose mean
            # is exactly 1 or 2 contributes the same value either way.
            v = vals.astype(np.float32)
            codes = np.where(v == 1.0, 1, np.where(v == 2.0, 2, 3)).astype(np.int8)
        codes = np.ascontiguousarray(codes, dtype=np.int8)
        col_off = np.zeros(self.m + 1, dtype=np.int64)
        np.cumsum(np.bincount(cols, minlength=self.m), out=col_off[1:])
        mean = np.ascontiguousarray(_host(mean), dtype=np.float32).reshape(-1)
        inv = np.ascontiguousarray(_host(inv), dtype=np.float32).reshape(-1)
        if mean.size != self.m or inv.size != self.m:
            raise ValueError(f"mean/inv must have m={self.m} entries.")
        self.h = C.c_void_p()
        stream = _lib.stream_ptr()
        with torch.cuda.device(device):
            _lib.check(self._lib.coherit_sparse_create_csc(
                self.n, self.m, col_off.ctypes.data, rows.ctypes.data, codes.ctypes.data,
                device.index, stream, C.byref(self.h)), "sparse shard")
            _lib.check(self._lib.coherit_sparse_set_stats(self.h, mean.ctypes.data,
                                                          inv.ctypes.data, stream), "shard stats")
        self.dev = device

    def apply(self, V, *, kv: bool):
        V, squeeze = as_rhs(V, self.dev)
        if V.shape[0] != self.n:
            raise ValueError(f"V has {V.shape[0]} rows, expected n={self.n}")
        k = int(V.shape[1])
        rows = self.n if kv else self.m
        out = torch.empty((rows, k), dtype=torch.float32, device=self.dev)
        if kv:
            _lib.check(self._lib.coherit_sparse_kv(self.h, V.data_ptr(), k, k, 1.0, 0.0,
                                                   out.data_ptr(), k, _lib.stream_ptr()), "kv")
        else:
            _lib.check(self._lib.coherit_sparse_xtv(self.h, V.data_ptr(), k, k, 1.0,
                                                    out.data_ptr(), k, _lib.stream_ptr()), "xtv")
        return out[:, 0] if squeeze else out

    def close(self):
        if self.h:
            self._lib.coherit_sparse_destroy(self.h)
            self.h = C.c_void_p()


def sparse_xtv_shard(V, *, m: int, mean, inv, csc_all_rows, csc_all_cols, csc_all_vals):
    """Standardised Z^T V of one rare-variant shard, shape (m, k) or (m,)
    (kv_impl.py:823-845)."""
    n = int(torch.as_tensor(V).shape[0])
    ts = _TransientSparse(n, m, mean, inv, csc_all_rows, csc_all_cols, csc_all_vals, _device(V))
    try:
        return ts.apply(V, kv=False)
    finally:
        ts.close()


def sparse_projected_core_atom_shard(U, *, m: int, mean, inv, csc_all_rows, csc_all_cols,
                                     csc_all_vals):
    """(Z^T U)^T (Z^T U) of one shard before m_eff scaling (kv_impl.py:848-870)."""
    if torch.as_tensor(U).ndim != 2:
        raise ValueError("sparse_projected_core_atom_shard expects U with shape (n, k).")
    blk = sparse_xtv_shard(U, m=m, mean=mean, inv=inv, csc_all_rows=csc_all_rows,
                           csc_all_cols=csc_all_cols, csc_all_vals=csc_all_vals)
    return blk.T @ blk


def sparse_kv_shard(V, *, n: int, m: int, sum_v=None, mean, b=None, inv_sq, row_b=None,
                    sum_a0_sq=None, csc_all_rows, csc_all_cols, csc_all_vals):
    """Unnormalised Z Z^T V of one shard (kv_impl.py:873-905).  The shard's
    inverse sds are sqrt(inv_sq); b, row_b, sum_a0_sq and sum_v are derived
    from the entries and statistics on the device and are accepted for call
    compatibility."""
    inv = np.sqrt(np.maximum(_host(inv_sq).astype(np.float32), 0.0)).astype(np.float32)
    ts = _TransientSparse(n, m, mean, inv, csc_all_rows, csc_all_cols, csc_all_vals, _device(V))
    try:
        return ts.apply(V, kv=True)
    finally:
        ts.close()


__all__ = [
    "sparse_xtv_shard",
    "sparse_projected_core_atom_shard",
    "sparse_kv_shard",
    "kv_impl_streamed",
    "kv_impl_snp_weighted_streamed",
    "xtv_impl_streamed",
    "xtv_impl_multi_streamed",
    "xtv_impl_multi_streamed_concat",
    "zxb_impl_streamed",
    "zxb_impl_same_stream_multi",
    "zxb_impl_multi_streamed",
    "kv_impl_multi_streamed_weighted",
    "kv_impl_multi_streamed_stacked",
    "kv_impl_partitioned_component",
    "kv_impl_partitioned_weighted",
    "kv_impl_partitioned_stacked",
    "build_projected_core_atom_streamed",
    "build_projected_core_atoms_multi_streamed",
    "build_projected_core_atoms_partitioned",
]
