"""Python mirror of caps-sa's in-memory suffix-array API over the GB300 C ABI.

Names and argument meanings follow the reference crate (caps-sa 0.7.0):

    build_in_memory(text)                               src/sample_sort.rs:97
    build_in_memory_with_opts(text, opts)               src/sample_sort.rs:106
    build_in_memory_with(text, lp, opts)                src/sample_sort.rs:118
    build_in_memory_for_positions(text, positions)      src/sample_sort.rs:143
    build_in_memory_for_positions_with_opts(...)        src/sample_sort.rs:152
    build_in_memory_for_positions_with(...)             src/sample_sort.rs:168
    build_in_memory_sample_sort(text, opts, emit)       src/ext_mem.rs:717
    try_build_in_memory_sample_sort(...)                src/ext_mem.rs:726
    build_in_memory_sample_sort_with(...)               src/ext_mem.rs:740
    build_in_memory_sample_sort_for_positions[_with]    src/ext_mem.rs:787, 824
    lcp / suffix_cmp / LcpDispatch                      src/lcp.rs:125-216
    PlainText / SegmentedText / BoundaryRank            src/limits.rs:107-336
    Opts / ExtMemOpts                                   src/sample_sort.rs:70-85,
                                                        src/ext_mem.rs:60-118

Texts are numpy arrays of uint8/uint16/uint32 (or CUDA tensors exposing
``data_ptr()``); the index type is chosen like the reference's generic
``I: Index`` (``index=np.uint32`` or ``np.uint64``).  Contract violations the
reference panics on raise ``ValueError``; emit aborts raise ``BuildError``.

Every call runs the CUDA library; there is no CPU fallback.  The library is
mapped on first use (a Context, or an attribute of ``lib``), which fails
loudly when it has not been built.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
import threading
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "_build", "libcapssa_gb300.so")

UNBOUNDED = (1 << 64) - 1


class Status(enum.IntEnum):
    OK = 0
    EINVAL = 1
    ENOMEM = 2
    ECUDA = 3
    ETIMEOUT = 4
    EEMIT = 5
    EUNSUPPORTED = 6


class CapsSaError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (Status(status).name, message))
        self.status = Status(status)


class BuildError(CapsSaError):
    """BuildError::Emit (src/ext_mem.rs:258-264): the emit callback aborted."""

    def __init__(self, status, message, inner=None):
        super().__init__(status, message)
        self.inner = inner


class BoundaryRank(enum.IntEnum):
    """src/limits.rs:113-123."""
    SHORTER_FIRST = 0
    LONGER_FIRST = 1


CDF_PARAMS = 257  # CAPSSA_CDF_PARAMS


class Partition(enum.IntEnum):
    AUTO = 0
    SPLITTERS = 1
    LEARNED = 2
    BISECT = 3


class Sampling(enum.IntEnum):
    """capssa_sampling: where the sample sort's splitter sample comes from."""
    AUTO = 0
    REFERENCE = 1
    PARTITION_FIRST = 2


class TieOrder(enum.IntEnum):
    """capssa_tie_order: order inside a tie class (SegmentedText, ShorterFirst)."""
    POSITION = 0   # ascending input order
    REFERENCE = 1  # as the reference's in-memory merge sort emits it


class _Limits(C.Structure):
    _fields_ = [("kind", C.c_int32), ("boundary", C.c_int32),
                ("ends", C.c_void_p), ("n_ends", C.c_uint64)]


class _Opts(C.Structure):
    _fields_ = [("max_context", C.c_uint64), ("subproblem_count", C.c_uint64),
                ("partition", C.c_int32), ("host_threads", C.c_int32),
                ("flags", C.c_uint64), ("sampling", C.c_int32), ("tie_order", C.c_int32),
                ("reserved", C.c_uint64 * 4)]




class _Stats(C.Structure):
    _fields_ = [("n_suffixes", C.c_uint64), ("key_symbols", C.c_uint32),
                ("key_bits_per_symbol", C.c_uint32), ("refine_rounds", C.c_uint32),
                ("partitions", C.c_uint32), ("refined_suffixes", C.c_uint64),
                ("max_partition", C.c_uint64), ("mispredicted", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("device_ms", C.c_double),
                ("h2d_ms", C.c_double), ("d2h_ms", C.c_double), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("keys_ms", C.c_double), ("sort_ms", C.c_double),
                ("refine_ms", C.c_double), ("finish_ms", C.c_double),
                ("sort_passes", C.c_uint32), ("sort_item_bytes", C.c_uint32),
                ("sort_pass_ms", C.c_double), ("partition_ms", C.c_double),
                ("train_ms", C.c_double), ("partition_probes", C.c_uint64),
                ("train_samples", C.c_uint32), ("model_loss", C.c_float),
                ("radix_items", C.c_uint32), ("sparse_subset", C.c_uint32),
                ("tie_classes", C.c_uint32), ("reserved_u32", C.c_uint32),
                ("tie_order_ms", C.c_double)]


class _Packer(C.Structure):
    _fields_ = [("bits", C.c_uint32), ("k", C.c_uint32), ("alphabet", C.c_uint32),
                ("identity", C.c_uint32), ("code", C.c_uint8 * 256)]


EMIT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_uint64), C.c_uint64)


class _Checksum128(C.Structure):
    _fields_ = [("count", C.c_uint64), ("lo", C.c_uint64), ("hi", C.c_uint64)]

_SYM = {np.dtype(np.uint8): "u8", np.dtype(np.uint16): "u16", np.dtype(np.uint32): "u32"}
_IDX = {np.dtype(np.uint32): "u32", np.dtype(np.uint64): "u64"}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libcapssa_gb300.so is not built (run caps-sa_gb300/build.py "
                          "or __graft_entry__.build()); there is no CPU fallback")
    L = C.CDLL(LIB_PATH)
    vp, u64, i32 = C.c_void_p, C.c_uint64, C.c_int32
    L.capssa_ctx_create.argtypes = [C.POINTER(vp), C.c_int]
    L.capssa_ctx_destroy.argtypes = [vp]
    L.capssa_ctx_last_error.argtypes = [vp]
    L.capssa_ctx_last_error.restype = C.c_char_p
    L.capssa_ctx_stats.argtypes = [vp, C.POINTER(_Stats)]
    L.capssa_ctx_workspace_bytes.argtypes = [vp]
    L.capssa_ctx_workspace_bytes.restype = u64
    L.capssa_ctx_trim.argtypes = [vp]
    L.capssa_cdf_grad.argtypes = [vp, vp, vp, vp, u64, vp, vp]
    L.capssa_selftest_bounded_wait.argtypes = [vp, C.c_uint32]
    L.capssa_cdf_train.argtypes = [vp, vp, vp, u64, i32, vp, vp]
    L.capssa_cdf_infer.argtypes = [vp, vp, vp, u64, vp]
    L.capssa_ctx_set_stream.argtypes = [vp, vp]
    L.capssa_opts_default.argtypes = [C.POINTER(_Opts)]
    for s in ("u8", "u16", "u32"):
        for i in ("u32", "u64"):
            getattr(L, "capssa_build_in_memory_%s_%s" % (s, i)).argtypes = [
                vp, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), vp]
            getattr(L, "capssa_build_in_memory_for_positions_%s_%s" % (s, i)).argtypes = [
                vp, vp, u64, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), vp]
            getattr(L, "capssa_build_in_memory_lcp_%s_%s" % (s, i)).argtypes = [
                vp, vp, u64, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), vp, vp]
            getattr(L, "capssa_merge_%s_%s" % (s, i)).argtypes = [
                vp, vp, u64, C.POINTER(_Limits), vp, vp, u64, vp, vp, u64, u64, vp, vp]
            getattr(L, "capssa_build_in_memory_for_filter_%s_%s" % (s, i)).argtypes = [
                vp, vp, u64, u64, u64, C.POINTER(_Limits), C.POINTER(_Opts), vp, vp]
            getattr(L, "capssa_build_batched_%s_%s" % (s, i)).argtypes = [
                vp, vp, vp, u64, C.POINTER(_Opts), vp]
        getattr(L, "capssa_build_in_memory_sample_sort_%s" % s).argtypes = [
            vp, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), EMIT_FN, vp]
        getattr(L, "capssa_build_in_memory_sample_sort_for_positions_%s" % s).argtypes = [
            vp, vp, u64, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), EMIT_FN, vp]
        getattr(L, "capssa_build_ext_mem_%s" % s).argtypes = [
            vp, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), EMIT_FN, vp]
        getattr(L, "capssa_build_ext_mem_for_positions_%s" % s).argtypes = [
            vp, vp, u64, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), EMIT_FN, vp]
        getattr(L, "capssa_build_ext_mem_for_filter_%s" % s).argtypes = [
            vp, vp, u64, u64, u64, C.POINTER(_Limits), C.POINTER(_Opts), EMIT_FN, vp, vp]
        getattr(L, "capssa_lcp_%s" % s).argtypes = [vp, vp, u64, vp, vp, u64, u64, vp]
        getattr(L, "capssa_sample_sort_plan_%s" % s).argtypes = [
            vp, vp, u64, vp, u64, C.POINTER(_Limits), C.POINTER(_Opts), vp, vp, vp]
        getattr(L, "capssa_suffix_cmp_%s" % s).argtypes = [
            vp, vp, u64, C.POINTER(_Limits), vp, vp, u64, u64, vp]
    L.capssa_checksum128_init.argtypes = [C.POINTER(_Checksum128)]
    L.capssa_checksum128_update.argtypes = [C.POINTER(_Checksum128), vp, u64]
    L.capssa_sa_lcp_records_u32.argtypes = [vp, vp, vp, u64, vp]
    L.capssa_sa_lcp_records_u64.argtypes = [vp, vp, vp, u64, vp]
    L.capssa_pack_params_u8.argtypes = [vp, vp, u64, i32, u64, C.POINTER(_Packer),
                                        C.POINTER(i32)]
    L.capssa_pack_keys_u8.argtypes = [vp, vp, u64, C.POINTER(_Packer), C.POINTER(_Limits), vp,
                                      u64, vp]
    for i in ("u32", "u64"):
        getattr(L, "capssa_seed_subarray_u8_%s" % i).argtypes = [
            vp, vp, u64, C.POINTER(_Packer), C.POINTER(_Limits), vp, vp, u64]
    return L


class _LazyLib:
    """The CUDA library, loaded on first use: importing the package (for
    example only for its workload generators or file formats) maps nothing."""

    _L = None

    def _get(self):
        if _LazyLib._L is None:
            _LazyLib._L = _load()
        return _LazyLib._L

    def __getattr__(self, name):
        return getattr(self._get(), name)


lib = _LazyLib()


# ------------------------------------------------------------------ providers

class PlainText:
    """lim_at(p) = n - p (src/limits.rs:125-156)."""

    def __init__(self, n: int, boundary: BoundaryRank = BoundaryRank.SHORTER_FIRST):
        self.n = int(n)
        self.boundary = BoundaryRank(boundary)

    def _c(self):
        return _Limits(0, int(self.boundary), None, 0)


class SegmentedText:
    """Segments at cumulative ends (src/limits.rs:158-336).  The STAR order of
    the reference's tests (lim_b.cmp(lim_a).then(p_a.cmp(p_b))) is
    ``boundary=BoundaryRank.LONGER_FIRST``."""

    def __init__(self, text_len: int, ends, boundary: BoundaryRank = BoundaryRank.SHORTER_FIRST):
        self.n = int(text_len)
        self.ends = np.ascontiguousarray(ends, dtype=np.uint64)
        self.boundary = BoundaryRank(boundary)
        if len(self.ends):
            if np.any(self.ends[1:] <= self.ends[:-1]):
                raise ValueError("SegmentedText::from_ends: ends must be strictly increasing")
            if int(self.ends[-1]) != self.n:
                raise ValueError("SegmentedText::from_ends: last end (%d) != text_len (%d)"
                                 % (int(self.ends[-1]), self.n))
        elif self.n != 0:
            raise ValueError("SegmentedText::from_ends: empty ends but text_len != 0")

    @classmethod
    def from_lengths(cls, text_len, lengths, boundary=BoundaryRank.SHORTER_FIRST):
        ends = np.cumsum(np.asarray(lengths, dtype=np.uint64), dtype=np.uint64)
        total = int(ends[-1]) if len(ends) else 0
        if total != int(text_len):
            raise ValueError("SegmentedText::from_lengths: per-segment lengths sum to %d but "
                             "text_len is %d" % (total, int(text_len)))
        return cls(text_len, ends, boundary)

    @classmethod
    def from_ends(cls, text_len, ends, boundary=BoundaryRank.SHORTER_FIRST):
        return cls(text_len, ends, boundary)

    def n_segments(self):
        return len(self.ends)

    def _c(self):
        return _Limits(1, int(self.boundary), self.ends.ctypes.data, len(self.ends))


@dataclass
class Opts:
    """src/sample_sort.rs:70-85; tie_order picks the order inside tie classes
    (the reference leaves it unpinned, src/sample_sort.rs:908-913)."""
    max_context: int = UNBOUNDED
    tie_order: TieOrder = TieOrder.POSITION


@dataclass
class ExtMemOpts:
    """The in-memory subset of src/ext_mem.rs:60-118."""
    max_context: int = UNBOUNDED
    subproblem_count: int = 0
    partition: Partition = Partition.AUTO
    host_threads: int = 0
    sampling: Sampling = Sampling.AUTO


def _copts(o) -> _Opts:
    c = _Opts()
    lib.capssa_opts_default(C.byref(c))
    if o is not None:
        c.max_context = int(getattr(o, "max_context", UNBOUNDED))
        c.subproblem_count = int(getattr(o, "subproblem_count", 0))
        c.partition = int(getattr(o, "partition", 0))
        c.host_threads = int(getattr(o, "host_threads", 0))
        c.flags = 0
        c.sampling = int(getattr(o, "sampling", 0))
        c.tie_order = int(getattr(o, "tie_order", 0))
    return c


# ------------------------------------------------------------------ buffers

def _is_cuda_tensor(a):
    return hasattr(a, "data_ptr") and getattr(getattr(a, "device", None), "type", "") == "cuda"


def _ptr_len_dtype(a):
    """(address, length, numpy dtype) of a numpy array or CUDA tensor."""
    if _is_cuda_tensor(a):
        import torch
        m = {torch.uint8: np.uint8, torch.int32: np.uint32, torch.int64: np.uint64}
        if hasattr(torch, "uint16"):
            m[torch.uint16] = np.uint16
        if hasattr(torch, "uint32"):
            m[torch.uint32] = np.uint32
        if hasattr(torch, "uint64"):
            m[torch.uint64] = np.uint64
        if not a.is_contiguous():
            raise ValueError("CUDA tensors must be contiguous")
        return a.data_ptr(), a.numel(), np.dtype(m[a.dtype])
    a = np.ascontiguousarray(a)
    return a.ctypes.data, len(a), a.dtype


def _text(text):
    if isinstance(text, (bytes, bytearray)):
        text = np.frombuffer(bytes(text), dtype=np.uint8)
    if not _is_cuda_tensor(text):
        text = np.ascontiguousarray(text)
    ptr, n, dt = _ptr_len_dtype(text)
    if dt not in _SYM:
        raise TypeError("symbols must be uint8, uint16 or uint32, got %s" % dt)
    return text, ptr, n, _SYM[dt]


# ------------------------------------------------------------------ context

class Context:
    """One GPU context (device memory cache + CUDA stream).  Not thread-safe."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = lib.capssa_ctx_create(C.byref(h), int(device))
        if st != 0:
            raise CapsSaError(st, "cannot create a context on CUDA device %d" % device)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib.capssa_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, inner=None):
        if st == 0:
            return
        msg = lib.capssa_ctx_last_error(self._h).decode()
        if st == Status.EINVAL:
            raise ValueError(msg)
        if st == Status.EEMIT:
            raise BuildError(st, msg, inner)
        raise CapsSaError(st, msg)

    def stats(self) -> dict:
        s = _Stats()
        lib.capssa_ctx_stats(self._h, C.byref(s))
        return {k: getattr(s, k) for k, _ in _Stats._fields_}

    def workspace_bytes(self) -> int:
        return int(lib.capssa_ctx_workspace_bytes(self._h))

    def trim(self):
        lib.capssa_ctx_trim(self._h)

    def set_stream(self, stream_ptr: int):
        self._check(lib.capssa_ctx_set_stream(self._h, C.c_void_p(stream_ptr)))

    # ---- builders

    def build_in_memory(self, text, lp=None, opts=None, index=np.uint32, out=None):
        """build_in_memory / _with_opts / _with (src/sample_sort.rs:97-127)."""
        text, tp, n, s = _text(text)
        idx = np.dtype(index)
        if lp is not None and lp.n != n:
            raise ValueError("limit provider length %d != text length %d" % (lp.n, n))
        if out is None:
            out = np.empty(n, dtype=idx)
        op, _, odt = _ptr_len_dtype(out)
        fn = getattr(lib, "capssa_build_in_memory_%s_%s" % (s, _IDX[odt]))
        lim = (lp or PlainText(n))._c()
        o = _copts(opts)
        self._check(fn(self._h, tp, n, C.byref(lim), C.byref(o), op))
        return out

    def build_in_memory_for_positions(self, text, positions, lp=None, opts=None, out=None):
        """build_in_memory_for_positions[_with[_opts]] (src/sample_sort.rs:143-206)."""
        text, tp, n, s = _text(text)
        if not _is_cuda_tensor(positions):
            positions = np.ascontiguousarray(positions)
            if positions.dtype not in (np.uint32, np.uint64):
                positions = positions.astype(np.uint64)
        pp, m, pdt = _ptr_len_dtype(positions)
        if out is None:
            out = np.empty(m, dtype=pdt)
        op, _, _ = _ptr_len_dtype(out)
        fn = getattr(lib, "capssa_build_in_memory_for_positions_%s_%s" % (s, _IDX[pdt]))
        lim = (lp or PlainText(n))._c()
        o = _copts(opts)
        self._check(fn(self._h, tp, n, pp, m, C.byref(lim), C.byref(o), op))
        return out

    def build_in_memory_lcp(self, text, positions=None, lp=None, opts=None, index=np.uint32):
        """Suffix array plus merge_sort's LCP postcondition
        (src/sample_sort.rs:208-216)."""
        text, tp, n, s = _text(text)
        if positions is not None:
            positions = np.ascontiguousarray(positions, dtype=index)
            m = len(positions)
            pp = positions.ctypes.data
        else:
            m, pp = n, None
        sa = np.empty(m, dtype=index)
        lcp = np.empty(m, dtype=index)
        fn = getattr(lib, "capssa_build_in_memory_lcp_%s_%s" % (s, _IDX[np.dtype(index)]))
        lim = (lp or PlainText(n))._c()
        o = _copts(opts)
        self._check(fn(self._h, tp, n, pp, m if positions is not None else 0, C.byref(lim),
                       C.byref(o), sa.ctypes.data, lcp.ctypes.data))
        return sa, lcp

    def try_build_in_memory_sample_sort(self, text, opts=None, emit=None, lp=None,
                                        positions=None):
        """try_build_in_memory_sample_sort[_for_positions]_with
        (src/ext_mem.rs:726-871).  `emit(batch: np.ndarray[u64])` is called in
        suffix order; raising from it aborts with BuildError."""
        text, tp, n, s = _text(text)
        err = {}

        def cb(user, ptr, length):
            try:
                arr = np.ctypeslib.as_array(ptr, shape=(length,))
                r = emit(arr)
                return 0 if r is None or r == 0 or r is True else 1
            except BaseException as e:  # the callback must not unwind through C
                err["e"] = e
                return 1

        cfn = EMIT_FN(cb)
        lim = (lp or PlainText(n))._c()
        o = _copts(opts)
        if positions is None:
            st = getattr(lib, "capssa_build_in_memory_sample_sort_%s" % s)(
                self._h, tp, n, C.byref(lim), C.byref(o), cfn, None)
        else:
            pos = np.ascontiguousarray(positions, dtype=np.uint64)
            st = getattr(lib, "capssa_build_in_memory_sample_sort_for_positions_%s" % s)(
                self._h, tp, n, pos.ctypes.data, len(pos), C.byref(lim), C.byref(o), cfn, None)
        self._check(st, err.get("e"))

    def build_in_memory_sample_sort(self, text, opts=None, emit=None, lp=None, positions=None):
        """build_in_memory_sample_sort[_with|_for_positions[_with]]
        (src/ext_mem.rs:717, 740, 787, 824); without `emit` the emitted
        positions are collected and returned."""
        if emit is None:
            chunks = []
            self.try_build_in_memory_sample_sort(text, opts, lambda b: chunks.append(b.copy()),
                                                 lp, positions)
            return np.concatenate(chunks) if chunks else np.zeros(0, dtype=np.uint64)
        self.try_build_in_memory_sample_sort(text, opts, emit, lp, positions)
        return None

    def try_build_ext_mem(self, text, opts=None, emit=None, lp=None, positions=None, keep=None):
        """try_build_ext_mem[_with], _for_positions[_with], _for_filter[_with]
        (src/ext_mem.rs:279-553).  `keep = (lo, hi)` selects the positions p
        with lo <= text[p] < hi (the filter source; a Python predicate cannot
        run on the device).  `emit(batch: np.ndarray[u64])` is called in
        suffix order; raising from it aborts with BuildError.  Returns the
        number of positions emitted."""
        err = {}

        def cb(user, ptr, length):
            try:
                arr = np.ctypeslib.as_array(ptr, shape=(length,))
                r = emit(arr)
                return 0 if r is None or r == 0 or r is True else 1
            except BaseException as e:  # the callback must not unwind through C
                err["e"] = e
                return 1

        cfn = EMIT_FN(cb)
        st, count = self._ext_mem_call(text, opts, lp, positions, keep, cfn, None)
        self._check(st, err.get("e"))
        return count

    def _ext_mem_call(self, text, opts, lp, positions, keep, cfn, user):
        """One capssa_build_ext_mem* call with a C emit callback: (status, count)."""
        if callable(keep):
            raise TypeError("keep must be a (lo, hi) symbol range: predicates run on the GPU")
        text, tp, n, s = _text(text)
        lim = (lp or PlainText(n))._c()
        o = _copts(opts)
        if keep is not None:
            if positions is not None:
                raise ValueError("give positions or keep, not both")
            lo, hi = keep
            m = C.c_uint64(0)
            st = getattr(lib, "capssa_build_ext_mem_for_filter_%s" % s)(
                self._h, tp, n, int(lo), int(hi), C.byref(lim), C.byref(o), cfn, user,
                C.byref(m))
            return st, int(m.value)
        if positions is None:
            return getattr(lib, "capssa_build_ext_mem_%s" % s)(
                self._h, tp, n, C.byref(lim), C.byref(o), cfn, user), n
        pos = np.ascontiguousarray(positions, dtype=np.uint64)
        st = getattr(lib, "capssa_build_ext_mem_for_positions_%s" % s)(
            self._h, tp, n, pos.ctypes.data, len(pos), C.byref(lim), C.byref(o), cfn, user)
        return st, len(pos)

    def build_ext_mem_to_file(self, path, text, opts=None, lp=None, positions=None, keep=None,
                              width=8):
        """The SA file of examples/caps_sa.rs:131-172: the emitted positions
        appended to `path` as little-endian u64 (width 8) or u32 (width 4)
        by the library's own C sink (no Python call per batch).  Returns the
        number of positions written."""
        if width not in (4, 8):
            raise ValueError("width must be 4 or 8")
        libc = C.CDLL(None)
        libc.fopen.restype = C.c_void_p
        libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
        libc.fclose.argtypes = [C.c_void_p]
        f = libc.fopen(os.fsencode(path), b"wb")
        if not f:
            raise OSError("cannot open %s for writing" % path)
        sink = C.cast(lib.capssa_emit_file_u64 if width == 8 else lib.capssa_emit_file_u32,
                      EMIT_FN)
        try:
            st, count = self._ext_mem_call(text, opts, lp, positions, keep, sink, C.c_void_p(f))
        finally:
            closed = libc.fclose(f)
        if st == Status.EEMIT:
            raise OSError("writing %s failed (disk full, or a position >= 2^32 for width 4)"
                          % path)
        self._check(st)
        if closed != 0:
            raise OSError("closing %s failed" % path)
        return count

    def ext_mem_checksum128(self, text, opts=None, lp=None, positions=None, keep=None):
        """(count, 128-bit checksum) of the emitted stream, computed by the
        library's C sink: the ruSTAR replay's regression signal
        (examples/rustar_segmented_bench.rs:236-245)."""
        ck = Checksum128()
        st, _ = self._ext_mem_call(text, opts, lp, positions, keep,
                                   C.cast(lib.capssa_emit_checksum128, EMIT_FN), C.byref(ck._c))
        self._check(st)
        return ck.count, ck.value

    def sa_lcp_records(self, sa, lcp):
        """SaLcp<I> bucket records (src/ext_bucket.rs:65-108) of an SA and its
        LCP array, interleaved on the GPU: a structured array with fields
        pos, lcp (little-endian u32 or u64, 8 or 16 bytes a record)."""
        sa = np.ascontiguousarray(sa)
        lcp = np.ascontiguousarray(lcp, dtype=sa.dtype)
        if sa.dtype not in (np.uint32, np.uint64) or len(lcp) != len(sa):
            raise ValueError("sa and lcp: equal-length u32 or u64 arrays")
        w = "<u4" if sa.dtype == np.uint32 else "<u8"
        out = np.empty(len(sa), dtype=[("pos", w), ("lcp", w)])
        fn = lib.capssa_sa_lcp_records_u32 if sa.dtype == np.uint32 else lib.capssa_sa_lcp_records_u64
        self._check(fn(self._h, sa.ctypes.data, lcp.ctypes.data, len(sa), out.ctypes.data))
        return out

    def build_ext_mem(self, text, opts=None, emit=None, lp=None, positions=None, keep=None):
        """build_ext_mem[_with|_for_positions[_with]|_for_filter[_with]]
        (src/ext_mem.rs:289, 315, 370, 399, 472, 503); without `emit` the
        emitted positions are collected and returned."""
        if emit is None:
            chunks = []
            self.try_build_ext_mem(text, opts, lambda b: chunks.append(b.copy()), lp, positions,
                                   keep)
            return np.concatenate(chunks) if chunks else np.zeros(0, dtype=np.uint64)
        self.try_build_ext_mem(text, opts, emit, lp, positions, keep)
        return None

    def build_in_memory_for_filter(self, text, lo, hi, lp=None, opts=None, index=np.uint64,
                                   out=None):
        """The positions p with lo <= text[p] < hi in suffix order: the filter
        source of build_ext_mem_for_filter (src/ext_mem.rs:927-1092), selected on
        the GPU.  Returns out[:m]."""
        text, tp, n, s = _text(text)
        lim = (lp or PlainText(n))._c()
        o = _copts(opts)
        idx = np.dtype(index) if out is None else _ptr_len_dtype(out)[2]
        fn = getattr(lib, "capssa_build_in_memory_for_filter_%s_%s" % (s, _IDX[idx]))
        m = C.c_uint64(0)
        if out is None:
            self._check(fn(self._h, tp, n, int(lo), int(hi), C.byref(lim), C.byref(o), None,
                           C.byref(m)))
            out = np.empty(int(m.value), dtype=idx)
        op, cap, _ = _ptr_len_dtype(out)
        self._check(fn(self._h, tp, n, int(lo), int(hi), C.byref(lim), C.byref(o), op,
                       C.byref(m)))
        if int(m.value) > cap:
            raise ValueError("output holds %d positions, %d kept" % (cap, int(m.value)))
        return out[:int(m.value)]

    def sample_sort_plan(self, text, opts=None, lp=None, positions=None):
        """The partition plan of build_in_memory_sample_sort (phases 1-3,
        src/ext_mem.rs:1191-1428): (p, pivots[p-1], partition sizes[p]).  With
        ExtMemOpts(partition=Partition.LEARNED) the partition comes from the
        learned CDF model with neighbour fixup (same plan)."""
        text, tp, n, s = _text(text)
        lim = (lp or PlainText(n))._c()
        o = _copts(opts)
        fn = getattr(lib, "capssa_sample_sort_plan_%s" % s)
        pp, m = None, 0
        if positions is not None:
            pos = np.ascontiguousarray(positions, dtype=np.uint64)
            pp, m = pos.ctypes.data, len(pos)
        p = C.c_uint64(0)
        self._check(fn(self._h, tp, n, pp, m, C.byref(lim), C.byref(o), C.byref(p), None, None))
        pv = np.zeros(max(int(p.value) - 1, 0) + 1, dtype=np.uint64)
        sz = np.zeros(max(int(p.value), 1), dtype=np.uint64)
        self._check(fn(self._h, tp, n, pp, m, C.byref(lim), C.byref(o), C.byref(p),
                       pv.ctypes.data, sz.ctypes.data))
        k = int(p.value)
        return k, pv[:max(k - 1, 0)], sz[:k]

    def selftest_bounded_wait(self, polls=4096):
        """Runs a bounded device wait that nothing satisfies; raises the
        CAPSSA_ETIMEOUT CapsSaError it must produce."""
        self._check(lib.capssa_selftest_bounded_wait(self._h, int(polls)))

    def cdf_grad(self, params, prefixes, targets):
        """(mean squared error, gradient) of the learned CDF model over the
        samples, from the GPU forward/backward kernels."""
        params = np.ascontiguousarray(params, dtype=np.float32)
        x = np.ascontiguousarray(prefixes, dtype=np.uint64)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(CDF_PARAMS, dtype=np.float32)
        loss = C.c_float(0)
        self._check(lib.capssa_cdf_grad(self._h, params.ctypes.data, x.ctypes.data,
                                        t.ctypes.data, len(x), g.ctypes.data, C.byref(loss)))
        return float(loss.value), g

    def cdf_infer(self, params, prefixes):
        """The model's outputs as the learned partition evaluates them (BF16
        weights, tensor-core layer 1, fp32 layer 2)."""
        params = np.ascontiguousarray(params, dtype=np.float32)
        x = np.ascontiguousarray(prefixes, dtype=np.uint64)
        y = np.zeros(len(x), dtype=np.float32)
        self._check(lib.capssa_cdf_infer(self._h, params.ctypes.data, x.ctypes.data, len(x),
                                         y.ctypes.data))
        return y

    def cdf_train(self, prefixes, targets, steps=300):
        """(trained parameters, final loss) after `steps` Adam steps on the GPU."""
        x = np.ascontiguousarray(prefixes, dtype=np.uint64)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        params = np.zeros(CDF_PARAMS, dtype=np.float32)
        loss = C.c_float(0)
        self._check(lib.capssa_cdf_train(self._h, x.ctypes.data, t.ctypes.data, len(x),
                                         int(steps), params.ctypes.data, C.byref(loss)))
        return params, float(loss.value)

    def build_batched(self, texts, offsets, index=np.uint32, opts=None, out=None):
        """Many independent texts: out[offsets[t]:offsets[t+1]] is the SA of
        texts[offsets[t]:offsets[t+1]] in local positions.  `out` may be a
        CUDA tensor (the result then stays on the device)."""
        text, tp, n, s = _text(texts)
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        if out is None:
            out = np.empty(n, dtype=index)
        op, _, odt = _ptr_len_dtype(out)
        fn = getattr(lib, "capssa_build_batched_%s_%s" % (s, _IDX[odt]))
        o = _copts(opts)
        self._check(fn(self._h, tp, offs.ctypes.data, len(offs) - 1, C.byref(o), op))
        return out

    # ---- primitives

    def lcp(self, text, p, q, max_ctx=UNBOUNDED):
        """LcpDispatch::lcp over arrays of pairs (src/lcp.rs:125-153)."""
        text, tp, n, s = _text(text)
        p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.uint64)
        q = np.ascontiguousarray(np.atleast_1d(q), dtype=np.uint64)
        out = np.empty(len(p), dtype=np.uint64)
        self._check(getattr(lib, "capssa_lcp_%s" % s)(self._h, tp, n, p.ctypes.data,
                                                       q.ctypes.data, len(p), int(max_ctx),
                                                       out.ctypes.data))
        return out

    def suffix_cmp(self, text, p, q, lp=None, max_ctx=UNBOUNDED):
        """LcpDispatch::suffix_cmp_with over arrays of pairs (src/lcp.rs:184-201)."""
        text, tp, n, s = _text(text)
        p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.uint64)
        q = np.ascontiguousarray(np.atleast_1d(q), dtype=np.uint64)
        out = np.empty(len(p), dtype=np.int8)
        lim = (lp or PlainText(n))._c()
        self._check(getattr(lib, "capssa_suffix_cmp_%s" % s)(
            self._h, tp, n, C.byref(lim), p.ctypes.data, q.ctypes.data, len(p), int(max_ctx),
            out.ctypes.data))
        return out

    def merge(self, text, x, lcp_x, y, lcp_y, lp=None, max_ctx=UNBOUNDED):
        """sample_sort::merge (src/sample_sort.rs:397-522)."""
        text, tp, n, s = _text(text)
        x = np.ascontiguousarray(x)
        dt = x.dtype
        y = np.ascontiguousarray(y, dtype=dt)
        lx = np.ascontiguousarray(lcp_x, dtype=dt)
        ly = np.ascontiguousarray(lcp_y, dtype=dt)
        z = np.empty(len(x) + len(y), dtype=dt)
        lz = np.empty_like(z)
        lim = (lp or PlainText(n))._c()
        self._check(getattr(lib, "capssa_merge_%s_%s" % (s, _IDX[dt]))(
            self._h, tp, n, C.byref(lim), x.ctypes.data, lx.ctypes.data, len(x), y.ctypes.data,
            ly.ctypes.data, len(y), int(max_ctx), z.ctypes.data, lz.ctypes.data))
        return z, lz

    def pack_params(self, text, policy=1, max_extra_bytes=0):
        """seed_params / Packer::new (src/pack.rs:103-176, 217-234)."""
        t = np.ascontiguousarray(text, dtype=np.uint8)
        pk = _Packer()
        avail = C.c_int32()
        self._check(lib.capssa_pack_params_u8(self._h, t.ctypes.data, len(t), int(policy),
                                              int(max_extra_bytes), C.byref(pk), C.byref(avail)))
        if not avail.value:
            return None
        return {"bits": pk.bits, "k": pk.k, "alphabet": pk.alphabet,
                "identity": pk.identity, "code": np.array(pk.code, dtype=np.uint8), "_c": pk}

    def pack_keys(self, text, params, positions, lp=None):
        """Packer::key_at_bounded per position (src/pack.rs:187-203)."""
        t = np.ascontiguousarray(text, dtype=np.uint8)
        pos = np.ascontiguousarray(positions, dtype=np.uint64)
        keys = np.empty(len(pos), dtype=np.uint64)
        lim = (lp or PlainText(len(t)))._c()
        self._check(lib.capssa_pack_keys_u8(self._h, t.ctypes.data, len(t), C.byref(params["_c"]),
                                            C.byref(lim), pos.ctypes.data, len(pos),
                                            keys.ctypes.data))
        return keys

    def seed_subarray(self, text, params, positions, lp=None, index=np.uint32):
        """seed_subarray (src/pack.rs:241-321) -> (sa, lcp)."""
        t = np.ascontiguousarray(text, dtype=np.uint8)
        sa = np.ascontiguousarray(positions, dtype=index).copy()
        lcp = np.zeros_like(sa)
        lim = (lp or PlainText(len(t)))._c()
        fn = getattr(lib, "capssa_seed_subarray_u8_%s" % _IDX[np.dtype(index)])
        self._check(fn(self._h, t.ctypes.data, len(t), C.byref(params["_c"]), C.byref(lim),
                       sa.ctypes.data, lcp.ctypes.data, len(sa)))
        return sa, lcp


# ------------------------------------------------------------------ free functions

_default = threading.local()


class Checksum128:
    """The order-sensitive 128-bit checksum of an emitted position stream
    (examples/rustar_segmented_bench.rs:236-245), kept by the library."""

    def __init__(self):
        self._c = _Checksum128()
        lib.capssa_checksum128_init(C.byref(self._c))

    def update(self, positions):
        p = np.ascontiguousarray(positions, dtype=np.uint64)
        lib.capssa_checksum128_update(C.byref(self._c), p.ctypes.data, len(p))
        return self

    @property
    def count(self) -> int:
        return int(self._c.count)

    @property
    def value(self) -> int:
        return (int(self._c.hi) << 64) | int(self._c.lo)


def default_context() -> Context:
    if getattr(_default, "ctx", None) is None:
        _default.ctx = Context(0)
    return _default.ctx


def build_in_memory(text, index=np.uint32):
    return default_context().build_in_memory(text, index=index)


def build_in_memory_with_opts(text, opts, index=np.uint32):
    return default_context().build_in_memory(text, None, opts, index)


def build_in_memory_with(text, lp, opts=None, index=np.uint32):
    return default_context().build_in_memory(text, lp, opts, index)


def build_in_memory_for_positions(text, positions):
    return default_context().build_in_memory_for_positions(text, positions)


def build_in_memory_for_positions_with_opts(text, positions, opts):
    return default_context().build_in_memory_for_positions(text, positions, None, opts)


def build_in_memory_for_positions_with(text, positions, lp, opts=None):
    return default_context().build_in_memory_for_positions(text, positions, lp, opts)


def build_in_memory_sample_sort(text, opts=None, emit=None):
    return default_context().build_in_memory_sample_sort(text, opts, emit)


def try_build_in_memory_sample_sort(text, opts, emit):
    return default_context().try_build_in_memory_sample_sort(text, opts, emit)


def build_in_memory_sample_sort_with(text, lp, opts=None, emit=None):
    return default_context().build_in_memory_sample_sort(text, opts, emit, lp)


def build_in_memory_sample_sort_for_positions(text, positions, opts=None, emit=None):
    return default_context().build_in_memory_sample_sort(text, opts, emit, None, positions)


def build_in_memory_sample_sort_for_positions_with(text, positions, lp, opts=None, emit=None):
    return default_context().build_in_memory_sample_sort(text, opts, emit, lp, positions)


def build_ext_mem(text, opts=None, emit=None):
    return default_context().build_ext_mem(text, opts, emit)


def try_build_ext_mem(text, opts, emit):
    return default_context().try_build_ext_mem(text, opts, emit)


def build_ext_mem_with(text, lp, opts=None, emit=None):
    return default_context().build_ext_mem(text, opts, emit, lp)


def build_ext_mem_for_positions(text, positions, opts=None, emit=None):
    return default_context().build_ext_mem(text, opts, emit, None, positions)


def build_ext_mem_for_positions_with(text, positions, lp, opts=None, emit=None):
    return default_context().build_ext_mem(text, opts, emit, lp, positions)


def build_ext_mem_for_filter(text, keep, opts=None, emit=None):
    return default_context().build_ext_mem(text, opts, emit, None, None, keep)


def build_ext_mem_for_filter_with(text, keep, lp, opts=None, emit=None):
    return default_context().build_ext_mem(text, opts, emit, lp, None, keep)


def lcp(text, p, q, max_ctx=UNBOUNDED):
    return int(default_context().lcp(text, p, q, max_ctx)[0])


def suffix_cmp(text, p, q, max_ctx=UNBOUNDED):
    return int(default_context().suffix_cmp(text, p, q, None, max_ctx)[0])
