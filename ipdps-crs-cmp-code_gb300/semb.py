"""ctypes binding of the GB300 semblance library (include/semb_gb300.h).

This is how Python callers (the tests and the benchmark) reach the CUDA path: every
call goes through the C ABI of _build/libsemb_gb300.so.  There is no fallback: if
the library is missing, `lib()` raises, and if no GPU is usable, Plan() raises
SembError(SEMB_E_NODEV).

Typical use, mirroring the reference's main():

    s = Survey.load("line.su", CMP, aph=800)          # su_gather + linearize
    with Plan(params(CMP, c0=1.98e-7, c1=1.77e-6, nc=101, aph=800, tau=0.002)) as p:
        p.upload(s.view())                              # device binning
        p.run()                                         # semblance + pick + stack
        ctr, sem, stk = p.download()
    s.write(p.params, ctr, sem, stk, out_dir)          # the reference's SU outputs
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# SEMB_CHECKED=1 in the environment selects the bounds-checked build of the same ABI
LIB_PATH = os.path.join(HERE, "_build", "libsemb_gb300_checked.so" if os.environ.get("SEMB_CHECKED") == "1"
                        else "libsemb_gb300.so")

CMP, CRS = 0, 1
PLAIN_F32, BATCHED = 0, 1
STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2
REPICK_OFF, REPICK_NEAR_TIES, REPICK_ALWAYS = 0, 1, 2
DM_ABS, DM_SIGNED = 0, 1
ABI_VERSION = 9
MAX_VARIANTS = 34   # SEMB_MAX_VARIANTS
MAX_BUCKETS = 4     # SEMB_MAX_BUCKETS

OK, E_ARG, E_IO, E_FORMAT, E_WINDOW, E_NOMEM, E_CUDA, E_TIMEOUT, E_STATE, E_NODEV, E_BOUNDS = range(11)

EXPORTS = [
    "semb_params_init", "semb_survey_load", "semb_survey_from_bytes", "semb_survey_view", "semb_survey_write",
    "semb_survey_free", "semb_plan_create", "semb_plan_upload", "semb_plan_stream", "semb_plan_run",
    "semb_plan_download", "semb_plan_download_attrs", "semb_survey_write_attr", "semb_plan_download_abc",
    "semb_survey_write_abc", "semb_plan_neighbours", "semb_neighbours_noalloc", "semb_plan_stats",
    "semb_plan_autotune", "semb_plan_buckets", "semb_plan_set_variant", "semb_plan_set_staging",
    "semb_plan_set_chunks", "semb_plan_chunk_times",
    "semb_plan_use_graph", "semb_plan_destroy",
    "semb_host_alloc", "semb_host_free", "semb_probe_fp32", "semb_selftest_wait", "semb_device_count",
    "semb_strerror", "semb_last_error", "semb_abi_version",
]


class SembParams(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("mode", C.c_int32),
        ("a0", C.c_double), ("a1", C.c_double), ("b0", C.c_double), ("b1", C.c_double),
        ("c0", C.c_double), ("c1", C.c_double),
        ("na", C.c_int32), ("nb", C.c_int32), ("nc", C.c_int32),
        ("aph", C.c_int32), ("apm", C.c_int32), ("storage", C.c_int32),
        ("tau", C.c_double), ("azimuth", C.c_double),
        ("repick", C.c_int32), ("repick_gap", C.c_float), ("dm_mode", C.c_int32),
        ("attrs", C.c_int32), ("ngen", C.c_int32),
    ]


class SembGatherView(C.Structure):
    _fields_ = [
        ("ncdps", C.c_int32), ("ns", C.c_int32), ("dt_us", C.c_int32), ("reserved", C.c_int32),
        ("ntraces", C.c_int64),
        ("cdp_end", C.c_void_p), ("cdp", C.c_void_p),
        ("gx", C.c_void_p), ("gy", C.c_void_p), ("sx", C.c_void_p), ("sy", C.c_void_p),
        ("scalco", C.c_void_p), ("samples", C.c_void_p),
    ]


class SembStats(C.Structure):
    _fields_ = [
        ("ms_search", C.c_double), ("ms_repick", C.c_double), ("ms_total", C.c_double), ("ms_upload", C.c_double),
        ("evals", C.c_int64), ("trace_evals", C.c_int64), ("repicked", C.c_int64), ("kernel_launches", C.c_int64),
        ("window", C.c_int32), ("max_aperture", C.c_int32), ("ncdps", C.c_int32), ("ns", C.c_int32),
        ("ncand", C.c_int32), ("grid_ctas", C.c_int32), ("ctas_per_sm", C.c_int32), ("sms", C.c_int32),
        ("variant", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class SembError(RuntimeError):
    def __init__(self, code: int, what: str, msg: str):
        super().__init__(f"{what}: {msg} (status {code})")
        self.code = code


_lib = None


def lib():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with build.py (nvcc, sm_103a)")
    L = C.CDLL(LIB_PATH)
    P, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    sig = {
        "semb_params_init": (None, [P, i32]),
        "semb_survey_load": (C.c_int, [C.c_char_p, i32, i32, P]),
        "semb_survey_from_bytes": (C.c_int, [P, i64, i32, i32, P]),
        "semb_survey_view": (C.c_int, [P, P]),
        "semb_survey_write": (C.c_int, [P, P, P, P, P, C.c_char_p]),
        "semb_survey_write_attr": (C.c_int, [P, C.c_char_p, P, C.c_char_p]),
        "semb_survey_free": (None, [P]),
        "semb_plan_create": (C.c_int, [P, i32, P]),
        "semb_plan_upload": (C.c_int, [P, P]),
        "semb_plan_run": (C.c_int, [P]),
        "semb_plan_stream": (C.c_int, [P, P, i32]),
        "semb_plan_download": (C.c_int, [P, P, P, P]),
        "semb_plan_download_attrs": (C.c_int, [P, P, P, P, P]),
        "semb_plan_download_abc": (C.c_int, [P, P, P, P]),
        "semb_survey_write_abc": (C.c_int, [P, P, P, P, P, P, C.c_char_p]),
        "semb_plan_neighbours": (C.c_int, [P, P, P, P]),
        "semb_plan_stats": (C.c_int, [P, P]),
        "semb_neighbours_noalloc": (C.c_int, [P, P, P, P, P, i32, i32, P, P, i64, P, P]),
        "semb_plan_autotune": (C.c_int, [P, P, P]),
        "semb_plan_buckets": (C.c_int, [P, P, P, P, P, P]),
        "semb_plan_set_variant": (C.c_int, [P, i32]),
        "semb_plan_set_staging": (C.c_int, [P, i32]),
        "semb_plan_set_chunks": (C.c_int, [P, i32]),
        "semb_plan_chunk_times": (C.c_int, [P, i32, P, P]),
        "semb_plan_use_graph": (C.c_int, [P, i32]),
        "semb_plan_destroy": (C.c_int, [P]),
        "semb_host_alloc": (C.c_int, [C.c_size_t, P]),
        "semb_host_free": (C.c_int, [P]),
        "semb_probe_fp32": (C.c_int, [i32, P]),
        "semb_selftest_wait": (C.c_int, [i32, i64, P]),
        "semb_device_count": (i32, []),
        "semb_strerror": (C.c_char_p, [C.c_int]),
        "semb_last_error": (C.c_char_p, []),
        "semb_abi_version": (i32, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if L.semb_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{LIB_PATH} has ABI {L.semb_abi_version()}, this binding expects {ABI_VERSION}: rebuild")
    _lib = L
    return L


def _check(rc: int, what: str) -> None:
    if rc != OK:
        L = lib()
        raise SembError(rc, what, f"{L.semb_strerror(rc).decode()}: {L.semb_last_error().decode()}")


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def params(method: int, mode: int = PLAIN_F32, storage: int = STORE_F16, repick: int = REPICK_NEAR_TIES,
           repick_gap: float = 1e-4, dm_mode: int = DM_ABS, attrs: int = 0, ngen: int = 0,
           **kw) -> SembParams:
    """Build semb_params from the reference's flag names (c0, c1, nc, aph, tau, and
    for CRS a0, a1, na, b0, b1, nb, apm, azimuth).  CMP values are rounded to float
    first, as the reference's stof does."""
    p = SembParams()
    lib().semb_params_init(C.byref(p), method)
    p.mode, p.storage, p.repick, p.repick_gap, p.dm_mode, p.attrs = mode, storage, repick, repick_gap, dm_mode, attrs
    p.ngen = ngen
    rnd = (lambda v: float(np.float32(v))) if method == CMP else float
    for k in ("a0", "a1", "b0", "b1", "c0", "c1", "tau", "azimuth"):
        if k in kw:
            setattr(p, k, rnd(kw[k]) if k != "azimuth" else float(kw[k]))
    for k in ("na", "nb", "nc", "aph", "apm"):
        if k in kw:
            setattr(p, k, int(kw[k]))
    return p


class GatherArrays:
    """A linearized gather held in numpy arrays (keeps them alive for the view)."""

    def __init__(self, cdp_end, ns, dt_us, gx, gy, sx, sy, scalco, samples, cdp=None):
        self.cdp_end = np.ascontiguousarray(cdp_end, dtype=np.int64)
        self.ns, self.dt_us = int(ns), int(dt_us)
        self.gx = np.ascontiguousarray(gx, dtype=np.int32)
        self.gy = np.ascontiguousarray(gy, dtype=np.int32)
        self.sx = np.ascontiguousarray(sx, dtype=np.int32)
        self.sy = np.ascontiguousarray(sy, dtype=np.int32)
        self.scalco = np.ascontiguousarray(scalco, dtype=np.int32)
        self.samples = samples if (isinstance(samples, np.ndarray) and samples.dtype == np.float32
                                   and samples.flags.c_contiguous) else np.ascontiguousarray(samples, np.float32)
        self.cdp = None if cdp is None else np.ascontiguousarray(cdp, dtype=np.int32)

    @property
    def ncdps(self) -> int:
        return len(self.cdp_end)

    def view(self) -> SembGatherView:
        v = SembGatherView()
        v.ncdps, v.ns, v.dt_us = self.ncdps, self.ns, self.dt_us
        v.ntraces = int(self.cdp_end[-1]) if self.ncdps else 0
        v.cdp_end, v.cdp = _ptr(self.cdp_end), _ptr(self.cdp)
        v.gx, v.gy, v.sx, v.sy = _ptr(self.gx), _ptr(self.gy), _ptr(self.sx), _ptr(self.sy)
        v.scalco, v.samples = _ptr(self.scalco), _ptr(self.samples)
        v._keep = self
        return v


class Survey:
    """An SU file grouped as the reference groups it (semb_survey_*)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def load(cls, path: str, method: int, aph: int) -> "Survey":
        h = C.c_void_p()
        _check(lib().semb_survey_load(str(path).encode(), method, int(aph), C.byref(h)), "semb_survey_load")
        return cls(h)

    @classmethod
    def from_bytes(cls, data: bytes | np.ndarray, method: int, aph: int) -> "Survey":
        buf = np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray)) else data.view(np.uint8)
        h = C.c_void_p()
        _check(lib().semb_survey_from_bytes(_ptr(buf), buf.size, method, int(aph), C.byref(h)),
               "semb_survey_from_bytes")
        return cls(h)

    def view(self) -> SembGatherView:
        v = SembGatherView()
        _check(lib().semb_survey_view(self._h, C.byref(v)), "semb_survey_view")
        v._keep = self
        return v

    def arrays(self) -> dict:
        """Copies of the linearized arrays (cdp_end, cdp, gx, ..., samples)."""
        v = self.view()
        n, nt = v.ncdps, v.ntraces

        def arr(ptr, cnt, dt):
            if cnt == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (cnt,)).copy()
        out = dict(ncdps=n, ns=v.ns, dt_us=v.dt_us, ntraces=nt,
                   cdp_end=arr(v.cdp_end, n, np.int64), cdp=arr(v.cdp, n, np.int32),
                   gx=arr(v.gx, nt, np.int32), gy=arr(v.gy, nt, np.int32), sx=arr(v.sx, nt, np.int32),
                   sy=arr(v.sy, nt, np.int32), scalco=arr(v.scalco, nt, np.int32))
        out["samples"] = arr(v.samples, nt * v.ns, np.float32).reshape(nt, v.ns)
        return out

    def write(self, p: SembParams, ctr, sem, stk, out_dir: str) -> None:
        ctr = np.ascontiguousarray(ctr, np.int32)
        sem = np.ascontiguousarray(sem, np.float32)
        stk = np.ascontiguousarray(stk, np.float32)
        _check(lib().semb_survey_write(self._h, C.byref(p), _ptr(ctr), _ptr(sem), _ptr(stk),
                                       str(out_dir).encode()), "semb_survey_write")

    def write_abc(self, a, b, c, sem, stk, out_dir: str) -> None:
        """crs.{a,b,c,coher,stack}.su from explicit parameter values (CRS-DE)."""
        arr = [np.ascontiguousarray(x, np.float32) for x in (a, b, c, sem, stk)]
        _check(lib().semb_survey_write_abc(self._h, *[_ptr(x) for x in arr], str(out_dir).encode()),
               "semb_survey_write_abc")

    def write_attr(self, name: str, data, out_dir: str) -> None:
        """One extra attribute file: a trace of ns samples per CDP (first-trace header)."""
        data = np.ascontiguousarray(data, np.float32)
        _check(lib().semb_survey_write_attr(self._h, name.encode(), _ptr(data), str(out_dir).encode()),
               "semb_survey_write_attr")

    def close(self) -> None:
        if self._h:
            lib().semb_survey_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """A search plan on one device (semb_plan_*)."""

    def __init__(self, p: SembParams, device: int = 0):
        self.params = p
        h = C.c_void_p()
        _check(lib().semb_plan_create(C.byref(p), int(device), C.byref(h)), "semb_plan_create")
        self._h = h
        self.ncdps = self.ns = 0

    def upload(self, view: SembGatherView) -> None:
        _check(lib().semb_plan_upload(self._h, C.byref(view)), "semb_plan_upload")
        self.ncdps, self.ns = view.ncdps, view.ns

    def stream(self, view: SembGatherView, nchunks: int = 4) -> None:
        """Upload and search in one call, the trace copies of CDP chunks overlapped
        with the search of earlier chunks (batched form)."""
        _check(lib().semb_plan_stream(self._h, C.byref(view), int(nchunks)), "semb_plan_stream")
        self.ncdps, self.ns = view.ncdps, view.ns

    def run(self) -> None:
        _check(lib().semb_plan_run(self._h), "semb_plan_run")

    def use_graph(self, on: bool = True) -> None:
        _check(lib().semb_plan_use_graph(self._h, 1 if on else 0), "semb_plan_use_graph")

    def download(self, ctr=None, sem=None, stk=None):
        n = self.ncdps * self.ns
        ctr = np.empty(n, np.int32) if ctr is None else ctr
        sem = np.empty(n, np.float32) if sem is None else sem
        stk = np.empty(n, np.float32) if stk is None else stk
        _check(lib().semb_plan_download(self._h, _ptr(ctr), _ptr(sem), _ptr(stk)), "semb_plan_download")
        return (ctr.reshape(self.ncdps, self.ns), sem.reshape(self.ncdps, self.ns), stk.reshape(self.ncdps, self.ns))

    def download_abc(self):
        """CRS-DE: the picked A, B, C per (CDP, t0) (C in s^2/m^2)."""
        n = self.ncdps * self.ns
        a, b, c = (np.empty(n, np.float32) for _ in range(3))
        _check(lib().semb_plan_download_abc(self._h, _ptr(a), _ptr(b), _ptr(c)), "semb_plan_download_abc")
        shp = (self.ncdps, self.ns)
        return a.reshape(shp), b.reshape(shp), c.reshape(shp)

    def download_attrs(self, batched: bool = True) -> dict:
        """Extra attributes of the last run: aperture traces per CDP and, for a batched
        plan made with attrs=1, the second-best candidate (sem2, idx2) and the FP64
        error of the pick (err64, -1 where not re-evaluated)."""
        n = self.ncdps * self.ns
        ap = np.empty(self.ncdps, np.int32)
        if not batched:
            _check(lib().semb_plan_download_attrs(self._h, None, None, None, _ptr(ap)), "semb_plan_download_attrs")
            return {"aperture": ap}
        sem2, idx2, err = np.empty(n, np.float32), np.empty(n, np.int32), np.empty(n, np.float32)
        _check(lib().semb_plan_download_attrs(self._h, _ptr(sem2), _ptr(idx2), _ptr(err), _ptr(ap)),
               "semb_plan_download_attrs")
        shp = (self.ncdps, self.ns)
        return {"aperture": ap, "sem2": sem2.reshape(shp), "idx2": idx2.reshape(shp), "err64": err.reshape(shp)}

    def neighbours(self):
        n = C.c_int64()
        _check(lib().semb_plan_neighbours(self._h, None, None, C.byref(n)), "semb_plan_neighbours")
        off = np.zeros(self.ncdps + 1, np.int32)
        lst = np.zeros(max(1, n.value), np.int32)
        _check(lib().semb_plan_neighbours(self._h, _ptr(off), _ptr(lst), None), "semb_plan_neighbours")
        return off, lst[:n.value]

    def autotune(self):
        """Pick the fastest search-kernel variant on a sample of this plan's tasks.
        Returns (chosen variant, [sample ms per variant, -1 when absent])."""
        v = C.c_int32()
        ms = (C.c_double * MAX_VARIANTS)()
        _check(lib().semb_plan_autotune(self._h, C.byref(v), ms), "semb_plan_autotune")
        return int(v.value), [float(x) for x in ms]

    def buckets(self) -> list:
        """Aperture buckets of the work queue: [(ap_lo, ap_hi, ntasks, variant), ...]."""
        n = C.c_int32()
        arrs = [(C.c_int32 * MAX_BUCKETS)() for _ in range(4)]
        _check(lib().semb_plan_buckets(self._h, C.byref(n), *arrs), "semb_plan_buckets")
        return [tuple(int(a[i]) for a in arrs) for i in range(n.value)]

    def set_variant(self, v: int) -> None:
        _check(lib().semb_plan_set_variant(self._h, int(v)), "semb_plan_set_variant")

    def set_chunks(self, cdps_per_chunk: int) -> None:
        """Run the batched grid search in chunks of contiguous CDPs, each chunk's
        work one CUDA graph (0: the whole survey at once)."""
        _check(lib().semb_plan_set_chunks(self._h, int(cdps_per_chunk)), "semb_plan_set_chunks")

    def chunk_times(self) -> list:
        """Device milliseconds of each chunk of the last chunked run."""
        n = C.c_int32()
        ms = (C.c_double * 4096)()
        _check(lib().semb_plan_chunk_times(self._h, 4096, ms, C.byref(n)), "semb_plan_chunk_times")
        return [float(ms[i]) for i in range(min(n.value, 4096))]

    def set_staging(self, max_samples: int) -> None:
        """Batched form: stage at most max_samples window samples per chunk (0:
        automatic); larger windows are read from the FP32 store in global memory."""
        _check(lib().semb_plan_set_staging(self._h, int(max_samples)), "semb_plan_set_staging")

    def stats(self) -> dict:
        s = SembStats()
        _check(lib().semb_plan_stats(self._h, C.byref(s)), "semb_plan_stats")
        return s.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().semb_plan_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """A numpy array in page-locked host memory (semb_host_alloc)."""

    def __init__(self, shape, dtype):
        self.dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * self.dtype.itemsize
        ptr = C.c_void_p()
        _check(lib().semb_host_alloc(max(nbytes, 1), C.byref(ptr)), "semb_host_alloc")
        self._ptr = ptr
        buf = (C.c_byte * max(nbytes, 1)).from_address(ptr.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self._ptr:
            self.array = None
            lib().semb_host_free(self._ptr)
            self._ptr = None


def neighbours_noalloc(gx_ptr, gy_ptr, sx_ptr, sy_ptr, scalco_ptr, ncdps: int, apm: int, off_ptr, list_ptr,
                       capacity: int, stream_ptr=None, check: bool = True):
    """semb_neighbours_noalloc on caller-owned device buffers (raw device pointers
    as ints).  Returns the list length; with check=False returns (status, length)
    instead of raising on a non-zero status."""
    n = C.c_int64(-1)
    rc = lib().semb_neighbours_noalloc(C.c_void_p(gx_ptr), C.c_void_p(gy_ptr), C.c_void_p(sx_ptr),
                                       C.c_void_p(sy_ptr), C.c_void_p(scalco_ptr), int(ncdps), int(apm),
                                       C.c_void_p(off_ptr), C.c_void_p(list_ptr), int(capacity), C.byref(n),
                                       C.c_void_p(stream_ptr) if stream_ptr else None)
    if not check:
        return int(rc), int(n.value)
    _check(rc, "semb_neighbours_noalloc")
    return int(n.value)


def probe_fp32_tflops(device: int = 0) -> float:
    v = C.c_double()
    _check(lib().semb_probe_fp32(int(device), C.byref(v)), "semb_probe_fp32")
    return float(v.value)


def selftest_wait(device: int = 0, limit_us: int = 20000) -> int:
    """1 when the bounded device-side wait gave up on a barrier nothing completes."""
    v = C.c_int32()
    _check(lib().semb_selftest_wait(int(device), int(limit_us), C.byref(v)), "semb_selftest_wait")
    return int(v.value)


def device_count() -> int:
    return int(lib().semb_device_count())
