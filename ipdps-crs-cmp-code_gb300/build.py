"""Build the GB300 semblance library and its command lines in-tree.

    python build.py            # -> _build/libsemb_gb300.so, _build/cmp-gb300, _build/crs-gb300

nvcc compiles every translation unit for sm_103a only (-gencode
arch=compute_103a,code=sm_103a), in parallel, then links one shared library with
the C ABI of include/semb_gb300.h and two executables that use it.  Host code is
built with -ffp-contract=off so that the reference's single-precision set-up
arithmetic (parameter grids, offsets) is reproduced on x86-64 and AArch64 alike.
Objects are rebuilt when a source or header is newer than them.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libsemb_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + INCLUDE, "-I" + CSRC]

LIB_SOURCES = ["su_io.cpp", "plan.cu", "launch.cu", "search_cmp_plain.cu", "search_cmp_fast.cu",
               "search_crs_plain.cu", "search_crs_fast.cu", "probe.cu", "noalloc.cu", "neighbours.cu", "de.cu"]
# the search kernels, compiled a second time with their window checks for the
# checked library (libsemb_gb300_checked.so, the same ABI)
SEARCH_SOURCES = ["search_cmp_plain.cu", "search_cmp_fast.cu", "search_crs_plain.cu", "search_crs_fast.cu"]
CHECKED_LIB = os.path.join(OUT, "libsemb_gb300_checked.so")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _deps() -> float:
    files = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, extra=()) -> str:
    obj = os.path.join(OUT, os.path.basename(src) + "".join(e.replace("-D", ".").replace("=", "") for e in extra) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= _deps():
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-x", "cu" if src.endswith(".cu") else "c++", "-c",
                                                  os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    jobs = [(s, ()) for s in LIB_SOURCES] + [(s, ("-DSEMB_CHECKED=1",)) for s in SEARCH_SOURCES] + [
        ("cli.cpp", ("-DSEMB_CLI_METHOD=0",)), ("cli.cpp", ("-DSEMB_CLI_METHOD=1",))]
    # the heaviest translation units (the search kernels) first
    order = sorted(range(len(jobs)), key=lambda i: not jobs[i][0].startswith("search_"))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        done = dict(zip(order, ex.map(lambda i: _compile(*jobs[i]), order)))
    objs = [done[i] for i in range(len(jobs))]
    nl, ns = len(LIB_SOURCES), len(SEARCH_SOURCES)
    lib_objs, checked_objs, cli_cmp, cli_crs = objs[:nl], objs[nl:nl + ns], objs[-2], objs[-1]
    checked_lib_objs = [o for o, src in zip(lib_objs, LIB_SOURCES) if src not in SEARCH_SOURCES] + checked_objs
    for out, parts in ((LIB, lib_objs), (CHECKED_LIB, checked_lib_objs)):
        newest = max(os.path.getmtime(o) for o in parts)
        if not os.path.exists(out) or os.path.getmtime(out) < newest:
            cmd = [nvcc()] + ARCH + ["-shared", "-o", out] + parts + ["-lcudart"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    for obj, name in ((cli_cmp, "cmp-gb300"), (cli_crs, "crs-gb300")):
        exe = os.path.join(OUT, name)
        if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(LIB), os.path.getmtime(obj)):
            cmd = [nvcc()] + ARCH + ["-o", exe, obj, "-L" + OUT, "-lsemb_gb300", "-Xlinker", "-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
