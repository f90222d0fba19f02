"""The C ABI surface (CPU): every function include/semb_gb300.h declares is
exported by the library, and calls that need no GPU behave as documented."""
import os
import re

import pytest

import semb

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "semb_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(semb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(semb_lib):
    names = declared_functions()
    assert len(names) >= 20
    lib = semb.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(semb.EXPORTS)


def test_versions_and_messages(semb_lib):
    lib = semb.lib()
    assert lib.semb_abi_version() == 7
    assert lib.semb_strerror(semb.OK) == b"ok"
    assert lib.semb_strerror(semb.E_NODEV) == b"no usable CUDA device"
    assert lib.semb_strerror(12345) == b"unknown error"


def test_params_defaults(semb_lib):
    p = semb.params(semb.CRS)
    assert p.method == semb.CRS and p.mode == semb.PLAIN_F32
    assert p.storage == semb.STORE_F16 and p.repick == semb.REPICK_NEAR_TIES
    assert abs(p.repick_gap - 1e-4) < 1e-9


def test_cmp_params_are_rounded_like_stof(semb_lib):
    p = semb.params(semb.CMP, c0=1.98e-7)
    import numpy as np
    assert p.c0 == float(np.float32(1.98e-7))
    q = semb.params(semb.CRS, c0=1.98e-7)
    assert q.c0 == 1.98e-7


@pytest.mark.skipif(semb.device_count() > 0, reason="a GPU is visible")
def test_no_device_is_reported_not_hidden(semb_lib):
    with pytest.raises(semb.SembError) as e:
        semb.Plan(semb.params(semb.CMP, c0=1e-7, c1=2e-7, nc=4, aph=100, tau=0.002))
    assert e.value.code == semb.E_NODEV


def test_plan_argument_checks_need_no_device(semb_lib):
    for bad in (dict(nc=0), dict(nc=4, tau=-1.0)):
        kw = dict(c0=1e-7, c1=2e-7, aph=100, tau=0.002)
        kw.update(bad)
        with pytest.raises(semb.SembError) as e:
            semb.Plan(semb.params(semb.CMP, **kw))
        assert e.value.code == semb.E_ARG
