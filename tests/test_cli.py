"""Command lines (CPU): the reference's parsing rules -- "-flag value" pairs, help and
exit status 1 on an unknown flag, "-h", a missing required flag or an odd number of
arguments (CMP/OpenMP/src/parser.cpp:44-103) -- and a clear failure without a GPU."""
import os
import subprocess

import pytest

import semb

BUILD = os.path.dirname(semb.LIB_PATH)
CMP = os.path.join(BUILD, "cmp-gb300")
CRS = os.path.join(BUILD, "crs-gb300")
CMP_ARGS = ["-c0", "1.98e-7", "-c1", "1.77e-6", "-nc", "8", "-aph", "600", "-tau", "0.002"]


def run(exe, args):
    return subprocess.run([exe] + args, capture_output=True, text=True)


@pytest.mark.parametrize("args", [[], ["-nc"], ["-zz", "1"], ["-h", "1"], ["-nc", "-h"], CMP_ARGS])
def test_help_and_exit_1(args):
    # the last case lacks the required -i
    r = run(CMP, args)
    assert r.returncode == 1
    assert r.stdout.startswith("Usage: ")
    assert "-c0: C0 constant" in r.stdout and "-tau: Tau constant" in r.stdout


def test_crs_help_lists_reference_flags():
    r = run(CRS, [])
    assert r.returncode == 1
    for flag in ("-a0", "-a1", "-na", "-b0", "-b1", "-nb", "-c0", "-c1", "-nc", "-aph", "-apm", "-azimuth",
                 "-tau", "-i", "-v"):
        assert f"  {flag}: " in r.stdout


def test_missing_input_file_fails_cleanly(tmp_path):
    r = run(CMP, CMP_ARGS + ["-i", str(tmp_path / "none.su")])
    assert r.returncode == 1
    assert r.stderr.startswith("[FAIL]") and "cannot open" in r.stderr


@pytest.mark.skipif(semb.device_count() > 0, reason="a GPU is visible")
def test_no_gpu_fails_without_cpu_fallback(tmp_path):
    import golden_cases as G
    meta, h, s, path = G.load("cmp_line")
    r = subprocess.run([CMP] + meta["args"] + ["-i", path], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1
    assert "no usable CUDA device" in r.stderr
    assert not (tmp_path / "cmp.coher.su").exists()
