"""Seismic Unix (SU) trace files: 240-byte little-endian header + ns float32 samples.

The header layout is the SEG-Y trace header as the reference declares it field by
field in su_trace (CRS/OpenMP/include/su_trace.hpp:42-125); a trace is read as the
raw header bytes followed by `ns` float32 samples (CRS/OpenMP/src/su_trace.cpp:37-51)
and written the same way (su_trace.cpp:55-66).  This module is the numpy view of
that format used by the synthetic generator, the tests and the benchmark; the
product's own loader is the C++ one in csrc/su_io.cpp.
"""
from __future__ import annotations

import numpy as np

# (name, numpy type) in file order.  Offsets follow from the sizes; the total is 240.
_FIELDS = [
    ("tracl", "<i4"), ("tracr", "<i4"), ("fldr", "<i4"), ("tracf", "<i4"),
    ("ep", "<i4"), ("cdp", "<i4"), ("cdpt", "<i4"),
    ("trid", "<i2"), ("nvs", "<i2"), ("nhs", "<i2"), ("duse", "<i2"),
    ("offset", "<i4"), ("gelev", "<i4"), ("selev", "<i4"), ("sdepth", "<i4"),
    ("gdel", "<i4"), ("sdel", "<i4"), ("swdep", "<i4"), ("gwdep", "<i4"),
    ("scalel", "<i2"), ("scalco", "<i2"),
    ("sx", "<i4"), ("sy", "<i4"), ("gx", "<i4"), ("gy", "<i4"),
    ("counit", "<i2"), ("wevel", "<i2"), ("swevel", "<i2"), ("sut", "<i2"),
    ("gut", "<i2"), ("sstat", "<i2"), ("gstat", "<i2"), ("tstat", "<i2"),
    ("laga", "<i2"), ("lagb", "<i2"), ("delrt", "<i2"), ("muts", "<i2"),
    ("mute", "<i2"), ("ns", "<u2"), ("dt", "<u2"),
    ("gain", "<i2"), ("igc", "<i2"), ("igi", "<i2"), ("corr", "<i2"),
    ("sfs", "<i2"), ("sfe", "<i2"), ("slen", "<i2"), ("styp", "<i2"),
    ("stas", "<i2"), ("stae", "<i2"), ("tatyp", "<i2"), ("afilf", "<i2"),
    ("afils", "<i2"), ("nofilf", "<i2"), ("nofils", "<i2"), ("lcf", "<i2"),
    ("hcf", "<i2"), ("lcs", "<i2"), ("hcs", "<i2"), ("year", "<i2"),
    ("day", "<i2"), ("hour", "<i2"), ("minute", "<i2"), ("sec", "<i2"),
    ("timbas", "<i2"), ("trwf", "<i2"), ("grnors", "<i2"), ("grnofr", "<i2"),
    ("grnlof", "<i2"), ("gaps", "<i2"), ("otrav", "<i2"),
    ("d1", "<f4"), ("f1", "<f4"), ("d2", "<f4"), ("f2", "<f4"),
    ("ungpow", "<f4"), ("unscale", "<f4"), ("ntr", "<i4"),
    ("mark", "<i2"), ("shortpad", "<i2"), ("unass", "<i2", (14,)),
]

HEADER_DTYPE = np.dtype(_FIELDS)
HEADER_SIZE = 240
assert HEADER_DTYPE.itemsize == HEADER_SIZE

# Byte offsets of the fields the semblance path reads (for C++/ctypes cross-checks).
OFFSETS = {name: HEADER_DTYPE.fields[name][1] for name in HEADER_DTYPE.names}


def trace_dtype(ns: int) -> np.dtype:
    """Structured dtype of one whole SU trace with `ns` samples."""
    return np.dtype([("hdr", HEADER_DTYPE), ("data", "<f4", (ns,))])


def empty_headers(n: int) -> np.ndarray:
    return np.zeros(n, dtype=HEADER_DTYPE)


def write_su(path, headers: np.ndarray, samples: np.ndarray) -> None:
    """Write traces (headers[i], samples[i, :]) to `path`.  headers['ns'] must equal
    samples.shape[1] for every trace."""
    samples = np.ascontiguousarray(samples, dtype="<f4")
    n, ns = samples.shape
    if len(headers) != n:
        raise ValueError("header/sample count mismatch")
    if n and not np.all(headers["ns"] == ns):
        raise ValueError("headers['ns'] disagrees with the sample array")
    rec = np.empty(n, dtype=trace_dtype(ns))
    rec["hdr"] = headers
    rec["data"] = samples
    with open(path, "wb") as f:
        rec.tofile(f)


def read_su(path):
    """Read a whole SU file whose traces all have the same ns.
    Returns (headers, samples[ntr, ns])."""
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size == 0:
        return empty_headers(0), np.zeros((0, 0), np.float32)
    if raw.size < HEADER_SIZE:
        raise ValueError(f"{path}: truncated SU header")
    first = raw[:HEADER_SIZE].view(HEADER_DTYPE)[0]
    ns = int(first["ns"])
    recsize = HEADER_SIZE + 4 * ns
    if raw.size % recsize:
        raise ValueError(f"{path}: size {raw.size} is not a whole number of {recsize}-byte traces")
    rec = raw.view(trace_dtype(ns))
    if not np.all(rec["hdr"]["ns"] == ns):
        raise ValueError(f"{path}: traces with different ns")
    return rec["hdr"].copy(), rec["data"].copy()
