"""On-disk formats and the library's host-side emit sinks (no GPU needed):
SA files, SaLcp records, the ruSTAR fixture, the 128-bit stream checksum."""
import ctypes
import os

import numpy as np
import pytest

capssa = pytest.importorskip("capssa")
from capssa import formats  # noqa: E402

FNV128_OFFSET = 0x6C62272E07BB014262B821756295C58D
FNV128_PRIME = 0x0000000001000000000000000000013B


def py_checksum(positions):
    """examples/rustar_segmented_bench.rs:236-245 in Python integers."""
    x = FNV128_OFFSET
    for p in positions:
        p = int(p)
        x ^= p
        x = (x * FNV128_PRIME) & ((1 << 128) - 1)
        x ^= p << 64
    return x


def test_sa_files_are_little_endian(tmp_path):
    p = tmp_path / "sa.u32"
    formats.write_sa(p, np.array([0x01020304, 7], dtype=np.uint32))
    assert p.read_bytes() == bytes([4, 3, 2, 1, 7, 0, 0, 0])
    assert formats.read_sa(p, 4).tolist() == [0x01020304, 7]
    q = tmp_path / "sa.u64"
    sa = np.array([5, 1 << 40, 3], dtype=np.uint64)
    formats.write_sa(q, sa)
    assert q.read_bytes()[:8] == bytes([5, 0, 0, 0, 0, 0, 0, 0])
    assert formats.read_sa(q).tolist() == sa.tolist()
    with pytest.raises(ValueError):
        formats.write_sa(tmp_path / "x", sa, width=4)
    (tmp_path / "odd").write_bytes(b"\0" * 7)
    with pytest.raises(ValueError):
        formats.read_sa(tmp_path / "odd", 8)


def test_sa_lcp_records_layout(tmp_path):
    for width in (4, 8):
        rec = np.zeros(3, dtype=formats.record_dtype(width))
        rec["pos"] = [2, 0, 1]
        rec["lcp"] = [0, 1, 3]
        p = tmp_path / ("rec%d" % width)
        formats.write_sa_lcp_records(p, rec)
        raw = p.read_bytes()
        assert len(raw) == 3 * 2 * width
        assert raw[:width] == (2).to_bytes(width, "little")
        assert raw[width:2 * width] == (0).to_bytes(width, "little")
        back = formats.read_sa_lcp_records(p, width)
        assert back["pos"].tolist() == [2, 0, 1] and back["lcp"].tolist() == [0, 1, 3]


def test_rustar_fixture_round_trip_and_checks(tmp_path):
    text = np.array([0, 1, 5, 2, 3, 5], dtype=np.uint8)
    formats.save_rustar_fixture(tmp_path / "fx", text, [3, 6])
    t, e = formats.load_rustar_fixture(tmp_path / "fx")
    assert t.tolist() == text.tolist() and e.tolist() == [3, 6]
    for bad in ([3, 5], [4, 3, 6], [0, 6]):
        d = tmp_path / ("bad%d" % len(os.listdir(tmp_path)))
        os.makedirs(d)
        (d / "text.bin").write_bytes(text.tobytes())
        (d / "ends.u64").write_bytes(np.array(bad, dtype="<u8").tobytes())
        with pytest.raises(ValueError):
            formats.load_rustar_fixture(d)


def test_checksum128_matches_restatement():
    rng = np.random.default_rng(3)
    pos = rng.integers(0, 1 << 40, 1000).astype(np.uint64)
    ck = capssa.Checksum128()
    ck.update(pos[:300]).update(pos[300:])  # batches compose
    assert ck.count == 1000
    assert ck.value == py_checksum(pos)
    assert capssa.Checksum128().value == FNV128_OFFSET


def test_c_file_sinks(tmp_path):
    """capssa_emit_file_u64 / _u32 called directly as emit callbacks."""
    libc = ctypes.CDLL(None)
    libc.fopen.restype = ctypes.c_void_p
    libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    libc.fclose.argtypes = [ctypes.c_void_p]
    lib = capssa.lib
    for width, fn in ((8, lib.capssa_emit_file_u64), (4, lib.capssa_emit_file_u32)):
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
        path = tmp_path / ("sink%d" % width)
        f = libc.fopen(os.fsencode(str(path)), b"wb")
        a = np.arange(10000, dtype=np.uint64) * 3
        assert fn(f, a[:6000].ctypes.data, 6000) == 0
        assert fn(f, a[6000:].ctypes.data, 4000) == 0
        if width == 4:
            big = np.array([1 << 33], dtype=np.uint64)
            assert fn(f, big.ctypes.data, 1) != 0  # does not fit: abort
        assert libc.fclose(f) == 0
        assert formats.read_sa(path, width).tolist() == a.tolist()
