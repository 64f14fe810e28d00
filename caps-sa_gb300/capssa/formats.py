"""On-disk formats around the suffix-array path.

* SA files: the positions as consecutive little-endian u32 or u64 values
  (examples/caps_sa.rs:131-139 writes u32, :147-189 u64), no header.
* SaLcp<I> bucket records: (pos, lcp) pairs, little-endian, 8 bytes for
  u32 and 16 for u64 (src/ext_bucket.rs:65-108).
* The ruSTAR replay fixture: a directory holding `text.bin` (the u8 text)
  and `ends.u64` (strictly increasing cumulative segment ends, little-endian
  u64, the last one equal to the text length) (bench/README.md:30-43).

Streaming writers that never hold the whole SA on the host are
Context.build_ext_mem_to_file and the C sinks capssa_emit_file_u64/_u32.
"""
from __future__ import annotations

import os

import numpy as np

_LE = {4: np.dtype("<u4"), 8: np.dtype("<u8")}


def write_sa(path, sa, width: int | None = None) -> int:
    """Write `sa` as little-endian values of `width` bytes (default: the
    array's own width, 4 for u32 and 8 for u64).  Returns the bytes written."""
    sa = np.asarray(sa)
    width = width or sa.dtype.itemsize
    if width not in _LE:
        raise ValueError("width must be 4 or 8")
    if width == 4 and len(sa) and int(sa.max()) > 0xFFFFFFFF:
        raise ValueError("a position does not fit in u32")
    data = np.ascontiguousarray(sa, dtype=_LE[width])
    with open(path, "wb") as f:
        f.write(data.tobytes())
    return data.nbytes


def read_sa(path, width: int = 8) -> np.ndarray:
    """An SA file of little-endian u32 (width 4) or u64 (width 8) values, in
    native byte order."""
    if width not in _LE:
        raise ValueError("width must be 4 or 8")
    size = os.path.getsize(path)
    if size % width:
        raise ValueError("%s: %d bytes is not a whole number of %d-byte entries"
                         % (path, size, width))
    return np.fromfile(path, dtype=_LE[width]).astype(np.uint32 if width == 4 else np.uint64)


def record_dtype(width: int) -> np.dtype:
    """dtype of one SaLcp record: pos then lcp, little-endian."""
    if width not in _LE:
        raise ValueError("width must be 4 or 8")
    return np.dtype([("pos", _LE[width]), ("lcp", _LE[width])])


def write_sa_lcp_records(path, records) -> int:
    records = np.ascontiguousarray(records)
    if records.dtype.names != ("pos", "lcp"):
        raise ValueError("records need fields pos, lcp")
    records = records.astype(record_dtype(records.dtype["pos"].itemsize))
    with open(path, "wb") as f:
        f.write(records.tobytes())
    return records.nbytes


def read_sa_lcp_records(path, width: int = 4) -> np.ndarray:
    dt = record_dtype(width)
    size = os.path.getsize(path)
    if size % dt.itemsize:
        raise ValueError("%s: %d bytes is not a whole number of %d-byte records"
                         % (path, size, dt.itemsize))
    return np.fromfile(path, dtype=dt)


def load_rustar_fixture(directory):
    """(text: u8 array, ends: u64 array) of a ruSTAR replay fixture, checked
    the way the replay checks it: ends strictly increasing, the last equal
    to the text length."""
    text = np.fromfile(os.path.join(directory, "text.bin"), dtype=np.uint8)
    ends_path = os.path.join(directory, "ends.u64")
    if os.path.getsize(ends_path) % 8:
        raise ValueError("ends.u64 is not a whole number of u64 values")
    ends = np.fromfile(ends_path, dtype="<u8").astype(np.uint64)
    if len(ends) == 0 or int(ends[-1]) != len(text):
        raise ValueError("the last segment end must equal the text length (%d)" % len(text))
    if len(ends) > 1 and not np.all(ends[1:] > ends[:-1]):
        raise ValueError("segment ends must be strictly increasing")
    if int(ends[0]) == 0:
        raise ValueError("segment ends must be positive")
    return text, ends


def save_rustar_fixture(directory, text, ends) -> None:
    text = np.ascontiguousarray(text, dtype=np.uint8)
    ends = np.ascontiguousarray(ends, dtype=np.uint64)
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "text.bin"), "wb") as f:
        f.write(text.tobytes())
    with open(os.path.join(directory, "ends.u64"), "wb") as f:
        f.write(ends.astype("<u8").tobytes())
    load_rustar_fixture(directory)  # the same checks as a reader
