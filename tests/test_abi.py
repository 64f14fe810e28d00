"""CPU checks of the C ABI: the library loads and exports every entry point
declared in include/capssa.h (no compute call: this machine may have no GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "capssa.h")
LIB = os.path.join(ROOT, "caps-sa_gb300", "_build", "libcapssa_gb300.so")


def declared_symbols():
    """Function names declared in the header, with the per-(S, I) macro
    families expanded."""
    src = open(HEADER).read()
    names = set(re.findall(r"^\s*(?:capssa_status|void|int|uint64_t|const char \*)\s*\*?\s*"
                           r"(capssa_[a-z0-9_]+)\s*\(", src, flags=re.M))
    sym = ["u8", "u16", "u32"]
    idx = ["u32", "u64"]
    fam_si = ["capssa_build_in_memory_%s_%s", "capssa_build_in_memory_for_positions_%s_%s",
              "capssa_build_in_memory_lcp_%s_%s", "capssa_merge_%s_%s",
              "capssa_build_batched_%s_%s", "capssa_build_in_memory_for_filter_%s_%s"]
    fam_s = ["capssa_build_in_memory_sample_sort_%s",
             "capssa_build_in_memory_sample_sort_for_positions_%s", "capssa_lcp_%s",
             "capssa_suffix_cmp_%s", "capssa_sample_sort_plan_%s", "capssa_build_ext_mem_%s",
             "capssa_build_ext_mem_for_positions_%s", "capssa_build_ext_mem_for_filter_%s"]
    for f in fam_si:
        for s in sym:
            for i in idx:
                names.add(f % (s, i))
    for f in fam_s:
        for s in sym:
            names.add(f % s)
    # macro templates themselves are not symbols
    return sorted(n for n in names if "##" not in n and not n.endswith("_"))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        import sys
        sys.path.insert(0, os.path.join(ROOT, "caps-sa_gb300"))
        import build as b
        b.build()
    return ctypes.CDLL(LIB)


def test_header_declares_expected_families():
    names = declared_symbols()
    assert "capssa_build_in_memory_u8_u32" in names
    assert "capssa_seed_subarray_u8_u64" in names
    assert "capssa_sample_sort_plan_u16" in names
    assert "capssa_cdf_grad" in names and "capssa_cdf_train" in names
    assert len(names) >= 55


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_defaults(lib):
    assert lib.capssa_abi_version() == 5

    class Opts(ctypes.Structure):
        _fields_ = [("max_context", ctypes.c_uint64), ("subproblem_count", ctypes.c_uint64),
                    ("partition", ctypes.c_int32), ("host_threads", ctypes.c_int32),
                    ("reserved", ctypes.c_uint64 * 6)]
    o = Opts()
    o.subproblem_count = 7
    lib.capssa_opts_default(ctypes.byref(o))
    assert o.max_context == (1 << 64) - 1 and o.subproblem_count == 0


def test_no_gpu_means_ecuda_not_a_cpu_fallback(lib):
    """Without a usable device the library refuses instead of computing on
    the host (this container has no GPU; on a GPU machine the context opens)."""
    h = ctypes.c_void_p()
    st = lib.capssa_ctx_create(ctypes.byref(h), 0)
    if st == 0:
        lib.capssa_ctx_destroy(h)
        pytest.skip("a CUDA device is present")
    assert st == 3  # CAPSSA_ECUDA
