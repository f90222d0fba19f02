"""Oracle wrappers (TEST INFRASTRUCTURE ONLY).

Used by tests/ as the checker of the CUDA path and by bench.py's CPU-baseline leg.
The product never imports this module.

* `gather()` restates the reference's SU ingest in numpy: the half-offset aperture
  filter and the grouping of traces by their `cdp` header in ascending order
  (CRS/OpenMP/src/su_gather.cpp:43-65), the per-CDP neighbour lists built from the
  first trace's midpoint (su_gather.cpp:70-87), and the flattening into arrays
  (su_gather::linearize, su_gather.cpp:94-127).  Float arithmetic is done in
  float32 or float64 exactly where the reference uses float or `real`.
* `cmp()` / `crs()` call the C restatement of the search (semb_oracle_body.h)
  through ctypes.
* `run_reference()` executes the reference's own programs built under _ref/ by the
  Makefile (only where the reference tree was available to build them).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsemb_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build_port()
        _lib = C.CDLL(LIB_PATH)
        P = C.c_void_p
        i32, f64 = C.c_int, C.c_double
        for sfx in ("_f32", "_f64"):
            f = getattr(_lib, "semb_oracle_cmp" + sfx)
            f.restype = i32
            f.argtypes = [i32, P, i32, i32, P, P, P, P, P, P, f64, f64, i32, f64, P, P, P, P, P, P, P, i32]
            f = getattr(_lib, "semb_oracle_crs" + sfx)
            f.restype = i32
            f.argtypes = [i32, P, i32, i32, P, P, P, P, P, P, P, P,
                          f64, f64, i32, f64, f64, i32, f64, f64, i32, f64,
                          P, P, P, P, P, P, P, P, P, P, i32]
        _lib.semb_oracle_max_threads.restype = i32
        _lib.semb_oracle_set_threads.argtypes = [i32]
        _lib.semb_oracle_set_dm.argtypes = [i32, f64]
        _lib.semb_oracle_set_t0.argtypes = [i32, i32]
        _lib.semb_oracle_set_top2.argtypes = [P]
        for sfx in ("_f32", "_f64"):
            f = getattr(_lib, "semb_oracle_crs_de" + sfx)
            f.restype = i32
            f.argtypes = [i32, P, i32, i32, P, P, P, P, P, P, P, P,
                          f64, f64, i32, f64, f64, i32, f64, f64, i32, f64, i32,
                          P, P, P, P, P, P, i32]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def parsed(method: str, v) -> float:
    """The value the reference's parser yields for a CLI number: std::stof for
    CMP (CMP/OpenMP/src/main.cpp:68-70), std::stod for CRS (CRS/OpenMP/src/main.cpp:85-91)."""
    s = v if isinstance(v, str) else repr(float(v))
    return float(np.float32(s)) if method == "cmp" else float(s)


def fscalco(scalco: np.ndarray) -> np.ndarray:
    """su_trace::fscalco (CRS/OpenMP/src/su_trace.cpp:102-107), float32."""
    s = scalco.astype(np.float32)
    out = np.where(scalco == 0, np.float32(1.0), s)
    neg = scalco < 0
    out[neg] = np.float32(1.0) / s[neg]
    return out.astype(np.float32)


def gather(headers: np.ndarray, samples: np.ndarray, method: str, aph: int, apm: int | None = None,
           real=np.float32) -> dict:
    """Restatement of su_gather + linearize.  `real` is the reference's `real` type
    (float32 for CMP as shipped, float64 for CRS as shipped)."""
    fs = fscalco(headers["scalco"])
    gx, sx = headers["gx"].astype(np.int32), headers["sx"].astype(np.int32)
    gy, sy = headers["gy"].astype(np.int32), headers["sy"].astype(np.int32)
    # halfoffset_x = fscalco() * (gx - sx) * 0.5, computed in float (su_trace.cpp:90-98)
    hx = (fs * (gx - sx).astype(np.float32)) * np.float32(0.5)
    hy = (fs * (gy - sy).astype(np.float32)) * np.float32(0.5)
    hxr, hyr = hx.astype(real), hy.astype(real)
    keep = ~((hxr * hxr + hyr * hyr) > real(int(aph) * int(aph)))
    idx = np.nonzero(keep)[0]
    if idx.size and not np.all(headers["ns"][idx] == headers["ns"][idx[0]]):
        raise ValueError("traces with different ns")
    cdp = headers["cdp"][idx]
    order = np.argsort(cdp, kind="stable")          # std::map order, file order inside a CDP
    tr = idx[order]
    cdp_sorted = headers["cdp"][tr]
    ucdp, counts = np.unique(cdp_sorted, return_counts=True)
    prefix = np.cumsum(counts).astype(np.int32)
    g = dict(
        method=method,
        trace_index=tr,                             # original file index of each linearized trace
        cdp_ids=ucdp.astype(np.int32),
        ntraces_by_cdp_id=prefix,
        ns=int(headers["ns"][tr[0]]) if tr.size else 0,
        dt_us=int(headers["dt"][tr[0]]) if tr.size else 0,
        samples=np.ascontiguousarray(samples[tr], dtype=np.float32),
        gx=gx[tr].copy(), gy=gy[tr].copy(), sx=sx[tr].copy(), sy=sy[tr].copy(),
        scalco=headers["scalco"][tr].astype(np.int32),
        first_header=headers[tr[np.concatenate([[0], prefix[:-1]])]] if tr.size else headers[:0],
    )
    if method == "crs":
        first = np.concatenate([[0], prefix[:-1]]).astype(np.int64)
        ft = tr[first]
        # midpoint_x = fscalco() * (gx + sx) * 0.5 in float (su_trace.cpp:70-80)
        mx = (fs[ft] * (gx[ft] + sx[ft]).astype(np.float32)) * np.float32(0.5)
        my = (fs[ft] * (gy[ft] + sy[ft]).astype(np.float32)) * np.float32(0.5)
        lim = np.float32(int(apm) * int(apm))
        offs, lists = [0], []
        for i in range(len(ucdp)):
            dx = mx - mx[i]
            dy = my - my[i]
            nb = np.nonzero((dx * dx + dy * dy) <= lim)[0].astype(np.int32)
            lists.append(nb)
            offs.append(offs[-1] + len(nb))
        g["nbr_off"] = np.asarray(offs, dtype=np.int32)
        g["nbr"] = np.concatenate(lists).astype(np.int32) if lists else np.zeros(0, np.int32)
    return g


def _list(cdps):
    if cdps is None:
        return None, 0
    a = np.ascontiguousarray(cdps, dtype=np.int32)
    return a, len(a)


def _sampling(L, ncdp, ns, t0_range, top2):
    """Set the t0 range and the top-2 gap output of the next search; returns the
    gap array (NaN where not evaluated) or None."""
    lo, hi = t0_range if t0_range is not None else (0, 0)
    L.semb_oracle_set_t0(int(lo), int(hi))
    gap = np.full(ncdp * ns, np.nan) if top2 else None
    L.semb_oracle_set_top2(_p(gap))
    return gap


def _unset(L):
    L.semb_oracle_set_t0(0, 0)
    L.semb_oracle_set_top2(None)


def cmp(g: dict, params: dict, precision: str = "f32", sem_all: bool = False, threads: int = 0,
        cdps=None, t0_range=None, top2: bool = False) -> dict:
    """CMP search of the gather (all CDPs, or only the CDP indices in `cdps`).
    t0_range=(lo, hi) evaluates only those output samples (other rows stay zero);
    top2=True adds out["top2"], the gap between the best and second-best candidate
    semblance per (CDP, t0)."""
    L = lib()
    if threads:
        L.semb_oracle_set_threads(threads)
    real = np.float32 if precision == "f32" else np.float64
    ncdp, ns = len(g["cdp_ids"]), g["ns"]
    nc = int(params["nc"])
    ctr = np.zeros(ncdp * ns, np.int32)
    strr = np.zeros(ncdp * ns, real)
    stk = np.zeros(ncdp * ns, real)
    outc = np.zeros(ncdp * ns, np.float32)
    sem = np.zeros(ncdp * ns * nc, real) if sem_all else None
    secs = np.zeros(1, np.float64)
    lst, nlst = _list(cdps)
    fn = getattr(L, "semb_oracle_cmp_" + precision)
    gap = _sampling(L, ncdp, ns, t0_range, top2)
    try:
        rc = fn(ncdp, _p(g["ntraces_by_cdp_id"]), ns, g["dt_us"], _p(g["samples"]),
                _p(g["gx"]), _p(g["gy"]), _p(g["sx"]), _p(g["sy"]), _p(g["scalco"]),
                parsed("cmp", params["c0"]), parsed("cmp", params["c1"]), nc, parsed("cmp", params["tau"]),
                _p(ctr), _p(strr), _p(stk), _p(outc), _p(sem), _p(secs), _p(lst), nlst)
    finally:
        _unset(L)
    if rc != 0:
        raise RuntimeError(f"oracle cmp failed: {rc}")
    out = dict(ctr=ctr.reshape(ncdp, ns), str=strr.reshape(ncdp, ns), stk=stk.reshape(ncdp, ns),
               c=outc.reshape(ncdp, ns), seconds=float(secs[0]))
    if sem_all:
        out["sem_all"] = sem.reshape(ncdp, ns, nc)
    if top2:
        out["top2"] = gap.reshape(ncdp, ns)
    return out


def crs(g: dict, params: dict, precision: str = "f64", sem_all: bool = False, threads: int = 0,
        cdps=None, dm_signed: bool = False, t0_range=None, top2: bool = False) -> dict:
    """CRS search of the gather (all CDPs, or only the CDP indices in `cdps`, with
    the neighbour lists of the whole gather).  `dm_signed` switches the midpoint
    displacement to the signed projection on params["azimuth"] (the library's
    SEMB_DM_SIGNED, which has no reference counterpart)."""
    L = lib()
    if threads:
        L.semb_oracle_set_threads(threads)
    L.semb_oracle_set_dm(1 if dm_signed else 0, float(params.get("azimuth", 0.0)))
    real = np.float32 if precision == "f32" else np.float64
    ncdp, ns = len(g["cdp_ids"]), g["ns"]
    na, nb, nc = int(params["na"]), int(params["nb"]), int(params["nc"])
    npar = na * nb * nc
    ctr = np.zeros(ncdp * ns, np.int32)
    strr = np.zeros(ncdp * ns, real)
    stk = np.zeros(ncdp * ns, real)
    oa, ob, oc = (np.zeros(ncdp * ns, np.float32) for _ in range(3))
    sem = np.zeros(ncdp * ns * npar, real) if sem_all else None
    secs = np.zeros(1, np.float64)
    nsem = np.zeros(1, np.int64)
    P = lambda k: parsed("crs", params[k])
    lst, nlst = _list(cdps)
    fn = getattr(L, "semb_oracle_crs_" + precision)
    gap = _sampling(L, ncdp, ns, t0_range, top2)
    try:
        rc = fn(ncdp, _p(g["ntraces_by_cdp_id"]), ns, g["dt_us"], _p(g["samples"]),
                _p(g["gx"]), _p(g["gy"]), _p(g["sx"]), _p(g["sy"]), _p(g["scalco"]),
                _p(g["nbr_off"]), _p(g["nbr"]),
                P("a0"), P("a1"), na, P("b0"), P("b1"), nb, P("c0"), P("c1"), nc, P("tau"),
                _p(ctr), _p(strr), _p(stk), _p(oa), _p(ob), _p(oc), _p(sem), _p(secs), _p(nsem), _p(lst), nlst)
    finally:
        _unset(L)
    if rc != 0:
        raise RuntimeError(f"oracle crs failed: {rc}")
    out = dict(ctr=ctr.reshape(ncdp, ns), str=strr.reshape(ncdp, ns), stk=stk.reshape(ncdp, ns),
               a=oa.reshape(ncdp, ns), b=ob.reshape(ncdp, ns), c=oc.reshape(ncdp, ns),
               seconds=float(secs[0]), n_semblance_traces=int(nsem[0]))
    if sem_all:
        out["sem_all"] = sem.reshape(ncdp, ns, npar)
    if top2:
        out["top2"] = gap.reshape(ncdp, ns)
    return out


def crs_de(g: dict, params: dict, ngen: int, precision: str = "f32", threads: int = 0, cdps=None,
           dm_signed: bool = False) -> dict:
    """CRS-DE search (differential evolution over A, B, C; the library's definition,
    restated in semb_oracle_body.h) of the gather: picked a, b, c, semblance, stack."""
    L = lib()
    if threads:
        L.semb_oracle_set_threads(threads)
    L.semb_oracle_set_dm(1 if dm_signed else 0, float(params.get("azimuth", 0.0)))
    real = np.float32 if precision == "f32" else np.float64
    ncdp, ns = len(g["cdp_ids"]), g["ns"]
    strr = np.zeros(ncdp * ns, real)
    stk = np.zeros(ncdp * ns, real)
    oa, ob, oc = (np.zeros(ncdp * ns, np.float32) for _ in range(3))
    P = lambda k: parsed("crs", params[k])
    lst, nlst = _list(cdps)
    fn = getattr(L, "semb_oracle_crs_de_" + precision)
    rc = fn(ncdp, _p(g["ntraces_by_cdp_id"]), ns, g["dt_us"], _p(g["samples"]),
            _p(g["gx"]), _p(g["gy"]), _p(g["sx"]), _p(g["sy"]), _p(g["scalco"]),
            _p(g["nbr_off"]), _p(g["nbr"]),
            P("a0"), P("a1"), int(params["na"]), P("b0"), P("b1"), int(params["nb"]), P("c0"), P("c1"),
            int(params["nc"]), P("tau"), int(ngen), _p(oa), _p(ob), _p(oc), _p(strr), _p(stk), _p(lst), nlst)
    if rc != 0:
        raise RuntimeError(f"oracle crs_de failed: {rc}")
    shp = (ncdp, ns)
    return dict(a=oa.reshape(shp), b=ob.reshape(shp), c=oc.reshape(shp), str=strr.reshape(shp), stk=stk.reshape(shp))


REF_OUTPUTS = {"cmp": ["c", "coher", "stack"], "crs": ["a", "b", "c", "coher", "stack"]}


def ref_binary(method: str, precision: str) -> str:
    shipped = {"cmp": "f32", "crs": "f64"}[method]
    name = f"{method}-omp2" + ("" if precision == shipped else "-" + {"f32": "fp32", "f64": "fp64"}[precision])
    return os.path.join(REF_DIR, name)


def have_reference() -> bool:
    return all(os.path.exists(ref_binary(m, p)) for m in ("cmp", "crs") for p in ("f32", "f64"))


def run_reference(method: str, precision: str, su_path: str, args: list, threads: int = 0,
                  workdir: str | None = None) -> dict:
    """Run the reference's own program on an SU file.  Returns {name: (headers, data)}
    for its output files plus the INFO line."""
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "ipdps-crs-cmp-code_gb300"))
    import su  # noqa: E402
    exe = ref_binary(method, precision)
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    tmp = workdir or tempfile.mkdtemp(prefix="semb_ref_")
    r = subprocess.run([exe] + list(args) + ["-i", os.path.abspath(su_path), "-v", "2"], cwd=tmp,
                       capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{exe} failed ({r.returncode}): {r.stdout}{r.stderr}")
    out = {"info": r.stdout.strip()}
    for k in REF_OUTPUTS[method]:
        out[k] = su.read_su(os.path.join(tmp, f"{method}.{k}.su"))
    return out
