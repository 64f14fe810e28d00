"""ctypes binding for the CPU restatement in capssa_oracle.c.

TEST INFRASTRUCTURE ONLY.  The tests, the smoke check and the CPU-baseline
leg of the benchmark load this module to check the GPU library against the
restated reference algorithm; the product never imports it.

Every function here forwards to a C function that cites the reference
(caps-sa 0.7.0) file:line it restates.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

UNBOUNDED = (1 << 64) - 1


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(LIB_PATH)
    for f in ("capssa_oracle.c", "cdf_oracle.c", "oracle_tmpl.h", "capssa_oracle.h"):
        if os.path.getmtime(os.path.join(HERE, f)) > t:
            return True
    return False


class _Limits(C.Structure):
    _fields_ = [
        ("n", C.c_uint64),
        ("segmented", C.c_int),
        ("longer_first", C.c_int),
        ("ends", C.POINTER(C.c_uint64)),
        ("n_ends", C.c_uint64),
        ("block_shift", C.c_uint32),
        ("dir", C.POINTER(C.c_uint32)),
        ("n_dir", C.c_uint64),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, u64, i = C.c_void_p, C.c_uint64, C.c_int
        L.or_limits_init.argtypes = [C.POINTER(_Limits), u64, i, i, vp, u64]
        L.or_limits_free.argtypes = [C.POINTER(_Limits)]
        L.or_lim_at.argtypes = [C.POINTER(_Limits), u64]
        L.or_lim_at.restype = u64
        L.or_limits_has_directory.argtypes = [C.POINTER(_Limits)]
        L.or_lcp.argtypes = [vp, u64, i, u64, u64, u64]
        L.or_lcp.restype = u64
        L.or_lcp_scalar.argtypes = [vp, u64, i, u64, u64, u64]
        L.or_lcp_scalar.restype = u64
        L.or_suffix_cmp.argtypes = [vp, i, C.POINTER(_Limits), u64, u64, u64]
        L.or_build_in_memory.argtypes = [vp, u64, i, i, vp, u64, C.POINTER(_Limits), u64, i,
                                         vp, vp]
        L.or_merge.argtypes = [vp, i, i, C.POINTER(_Limits), vp, u64, vp, vp, u64, vp, u64,
                               vp, vp]
        L.or_sample_sort.argtypes = [vp, u64, i, vp, u64, C.POINTER(_Limits), u64, u64, i,
                                     vp, vp, vp, vp, vp, vp]
        L.or_pack_params.argtypes = [vp, u64, i, u64, vp, vp, vp, vp]
        L.or_pack_keys.argtypes = [vp, u64, vp, C.c_uint32, C.c_uint32, C.c_uint32, i,
                                   C.POINTER(_Limits), vp, u64, vp]
        L.or_seed_subarray.argtypes = [vp, u64, i, C.POINTER(_Limits), vp, C.c_uint32,
                                       C.c_uint32, C.c_uint32, vp, vp, u64]
        L.or_brute_sa.argtypes = [vp, u64, i, C.POINTER(_Limits), u64, vp, u64, vp]
        L.or_max_threads.restype = i
        L.or_adjacent_cmp.argtypes = [vp, i, C.POINTER(_Limits), i, vp, u64, u64, vp]
        L.or_cdf_forward.argtypes = [vp, u64]
        L.or_cdf_forward.restype = C.c_double
        L.or_cdf_loss_grad.argtypes = [vp, vp, vp, u64, vp]
        L.or_cdf_loss_grad.restype = C.c_double
        L.or_cdf_features.argtypes = [u64, vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Limits:
    """PlainText / SegmentedText / STAR-order provider (src/limits.rs)."""

    def __init__(self, n, ends=None, longer_first=False):
        self._ends = None if ends is None else np.ascontiguousarray(ends, dtype=np.uint64)
        self.s = _Limits()
        ptr = None if self._ends is None else self._ends.ctypes.data_as(C.c_void_p)
        rc = lib().or_limits_init(C.byref(self.s), int(n), int(ends is not None),
                                  int(longer_first), ptr,
                                  0 if self._ends is None else len(self._ends))
        if rc != 0:
            raise ValueError("invalid segment ends (rc=%d)" % rc)

    def __del__(self):
        try:
            lib().or_limits_free(C.byref(self.s))
        except Exception:
            pass

    @property
    def ref(self):
        return C.byref(self.s)

    def lim_at(self, p):
        return int(lib().or_lim_at(self.ref, int(p)))

    def has_directory(self):
        return bool(lib().or_limits_has_directory(self.ref))


def _text(text):
    t = np.ascontiguousarray(text)
    if t.dtype not in (np.uint8, np.uint16, np.uint32):
        raise TypeError("symbols must be u8/u16/u32")
    return t


def lcp(text, p, q, max_ctx=UNBOUNDED):
    t = _text(text)
    return int(lib().or_lcp(_ptr(t), len(t), t.itemsize, int(p), int(q), int(max_ctx)))


def lcp_scalar(text, p, q, max_ctx=UNBOUNDED):
    t = _text(text)
    return int(lib().or_lcp_scalar(_ptr(t), len(t), t.itemsize, int(p), int(q), int(max_ctx)))


def suffix_cmp(text, p, q, limits=None, max_ctx=UNBOUNDED):
    t = _text(text)
    lp = limits or Limits(len(t))
    return int(lib().or_suffix_cmp(_ptr(t), t.itemsize, lp.ref, int(p), int(q), int(max_ctx)))


def build_in_memory(text, positions=None, limits=None, max_ctx=UNBOUNDED, index=np.uint32,
                    threads=0, with_lcp=False):
    """build_in_memory_for_positions_with (src/sample_sort.rs:168-206)."""
    t = _text(text)
    lp = limits or Limits(len(t))
    if positions is None:
        positions = np.arange(len(t), dtype=index)
    pos = np.ascontiguousarray(positions, dtype=index)
    out = np.empty_like(pos)
    lcp_out = np.empty_like(pos) if with_lcp else None
    rc = lib().or_build_in_memory(_ptr(t), len(t), t.itemsize, pos.itemsize, _ptr(pos), len(pos),
                                  lp.ref, int(max_ctx), int(threads), _ptr(out), _ptr(lcp_out))
    if rc != 0:
        raise ValueError("oracle build rc=%d" % rc)
    return (out, lcp_out) if with_lcp else out


def merge(text, x, lcp_x, y, lcp_y, limits=None, max_ctx=UNBOUNDED):
    """sample_sort::merge (src/sample_sort.rs:397-522)."""
    t = _text(text)
    lp = limits or Limits(len(t))
    x = np.ascontiguousarray(x)
    dt = x.dtype
    y = np.ascontiguousarray(y, dtype=dt)
    lx = np.ascontiguousarray(lcp_x, dtype=dt)
    ly = np.ascontiguousarray(lcp_y, dtype=dt)
    z = np.empty(len(x) + len(y), dtype=dt)
    lz = np.empty_like(z)
    rc = lib().or_merge(_ptr(t), t.itemsize, dt.itemsize, lp.ref, _ptr(x), len(x), _ptr(lx),
                        _ptr(y), len(y), _ptr(ly), int(max_ctx), _ptr(z), _ptr(lz))
    if rc != 0:
        raise ValueError("oracle merge rc=%d" % rc)
    return z, lz


def sample_sort(text, positions=None, limits=None, max_ctx=UNBOUNDED, subproblem_count=0,
                threads=0):
    """build_in_memory_sample_sort[_for_positions]_with (src/ext_mem.rs:651-871).

    Returns (emitted positions u64, p, pivots, partition sizes)."""
    t = _text(text)
    lp = limits or Limits(len(t))
    pos = None if positions is None else np.ascontiguousarray(positions, dtype=np.uint64)
    m = len(t) if pos is None else len(pos)
    out = np.empty(m, dtype=np.uint64)
    p = C.c_uint64(0)
    pivots = np.zeros(max(m, 1), dtype=np.uint64)
    sizes = np.zeros(max(m, 1), dtype=np.uint64)
    rc = lib().or_sample_sort(_ptr(t), len(t), t.itemsize, _ptr(pos), m, lp.ref, int(max_ctx),
                              int(subproblem_count), int(threads), _ptr(out), C.byref(p),
                              _ptr(pivots), _ptr(sizes), None, None)
    if rc != 0:
        raise ValueError("oracle sample sort rc=%d" % rc)
    pv = int(p.value)
    return out, pv, pivots[: max(pv - 1, 0)].copy(), sizes[:pv].copy()


def pack_params(text, policy=1, max_extra_bytes=0):
    """seed_params / Packer::new (src/pack.rs:103-176, 217-234)."""
    t = np.ascontiguousarray(text, dtype=np.uint8)
    bits, k, alpha = C.c_uint32(), C.c_uint32(), C.c_uint32()
    code = np.zeros(256, dtype=np.uint8)
    ok = lib().or_pack_params(_ptr(t), len(t), int(policy), int(max_extra_bytes), C.byref(bits),
                              C.byref(k), C.byref(alpha), _ptr(code))
    if not ok:
        return None
    return {"bits": bits.value, "k": k.value, "alphabet": alpha.value, "code": code}


def pack_keys(text, params, positions, limits=None):
    t = np.ascontiguousarray(text, dtype=np.uint8)
    lp = limits or Limits(len(t))
    pos = np.ascontiguousarray(positions, dtype=np.uint64)
    keys = np.empty(len(pos), dtype=np.uint64)
    lib().or_pack_keys(_ptr(t), len(t), _ptr(params["code"]), params["bits"], params["k"],
                       params["alphabet"], int(lp.s.longer_first), lp.ref, _ptr(pos), len(pos),
                       _ptr(keys))
    return keys


def seed_subarray(text, params, positions, limits=None, index=np.uint32):
    """seed_subarray (src/pack.rs:241-321) -> (sa, lcp)."""
    t = np.ascontiguousarray(text, dtype=np.uint8)
    lp = limits or Limits(len(t))
    sa = np.ascontiguousarray(positions, dtype=index).copy()
    lcp_out = np.zeros_like(sa)
    rc = lib().or_seed_subarray(_ptr(t), len(t), sa.itemsize, lp.ref, _ptr(params["code"]),
                                params["bits"], params["k"], params["alphabet"], _ptr(sa),
                                _ptr(lcp_out), len(sa))
    if rc != 0:
        raise ValueError("oracle seed rc=%d" % rc)
    return sa, lcp_out


def brute_sa(text, positions=None, limits=None, max_ctx=UNBOUNDED):
    """Full-comparator sort, ties by position (src/sample_sort.rs:643-647, 1021-1040)."""
    t = _text(text)
    lp = limits or Limits(len(t))
    pos = None if positions is None else np.ascontiguousarray(positions, dtype=np.uint64)
    m = len(t) if pos is None else len(pos)
    out = np.empty(m, dtype=np.uint64)
    rc = lib().or_brute_sa(_ptr(t), len(t), t.itemsize, lp.ref, int(max_ctx), _ptr(pos), m,
                           _ptr(out))
    if rc != 0:
        raise ValueError("oracle brute rc=%d" % rc)
    return out


def adjacent_cmp(text, sa, limits=None, max_ctx=UNBOUNDED):
    """Sign (-1, 0, 1) of suffix_cmp_with for every adjacent pair of sa."""
    t = _text(text)
    lp = limits or Limits(len(t))
    a = np.ascontiguousarray(sa)
    if a.dtype not in (np.uint32, np.uint64):
        a = a.astype(np.uint64)
    out = np.zeros(max(len(a) - 1, 0), dtype=np.int8)
    lib().or_adjacent_cmp(_ptr(t), t.itemsize, lp.ref, a.itemsize, _ptr(a), len(a),
                          int(max_ctx), _ptr(out))
    return out


def canonical_ties(sa, cmp):
    """sa with every tie class (a run of adjacent pairs comparing equal)
    sorted by position: the reference leaves the order inside a class
    unpinned under SegmentedText's default boundary order.  Only the members
    of classes of two or more are reordered."""
    a = np.array(sa, copy=True)
    tie = np.asarray(cmp) == 0
    if len(a) < 2 or not tie.any():
        return a
    mem = np.zeros(len(a), dtype=bool)
    at = np.nonzero(tie)[0]
    mem[at] = True
    mem[at + 1] = True
    sel = np.nonzero(mem)[0]
    start = np.ones(len(sel), dtype=bool)  # a member opens a class unless tied to its left
    inner = sel > 0
    start[inner] = ~tie[sel[inner] - 1]
    run = np.cumsum(start)
    vals = a[sel]
    a[sel] = vals[np.lexsort((vals, run))]
    return a


def max_threads():
    return int(lib().or_max_threads())


# ---------------------------------------------------------------- learned CDF model

CDF_HIDDEN = 64
CDF_PARAMS = 4 * CDF_HIDDEN + 1


def cdf_features(prefix):
    """The model's two float inputs for one 64-bit packed prefix."""
    f = np.zeros(2, dtype=np.float32)
    lib().or_cdf_features(int(prefix), _ptr(f))
    return f


def cdf_forward(params, prefixes):
    """Model output per prefix (double accumulation)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    return np.array([lib().or_cdf_forward(_ptr(params), int(x)) for x in prefixes])


def cdf_loss_grad(params, prefixes, targets):
    """(mean squared error, gradient of it w.r.t. the 257 parameters)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    prefixes = np.ascontiguousarray(prefixes, dtype=np.uint64)
    targets = np.ascontiguousarray(targets, dtype=np.float32)
    grad = np.zeros(CDF_PARAMS, dtype=np.float64)
    loss = lib().or_cdf_loss_grad(_ptr(params), _ptr(prefixes), _ptr(targets),
                                  len(prefixes), _ptr(grad))
    return loss, grad
