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
    assert lib.semb_abi_version() == semb.ABI_VERSION == 9
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


def test_extension_parameters_are_checked_before_the_device(semb_lib):
    crs = dict(a0=-1e-3, a1=1e-3, na=2, b0=-1e-7, b1=1e-7, nb=2, c0=1e-7, c1=2e-7, nc=2, aph=100, apm=25,
               tau=0.002)
    bad = [
        (semb.CRS, dict(dm_mode=7), crs),                                  # unknown displacement mode
        (semb.CRS, dict(attrs=2), crs),                                    # attrs is 0 or 1
        (semb.CRS, dict(ngen=-1), crs),                                    # negative generations
        (semb.CRS, dict(ngen=3, mode=semb.BATCHED), crs),                  # CRS-DE is plain-form only
        (semb.CMP, dict(ngen=3), dict(c0=1e-7, c1=2e-7, nc=4, aph=100, tau=0.002)),   # CRS only
        (semb.CRS, dict(ngen=3), dict(crs, na=7, nb=7, nc=7)),             # population 343 > 256
        (semb.CRS, dict(storage=5), crs),                                  # unknown storage
        (semb.CRS, dict(repick=3), crs),                                   # unknown re-pick mode
        (semb.CRS, {}, dict(crs, azimuth=float("nan"))),                   # azimuth must be finite
        (semb.CRS, {}, dict(crs, na=0)),                                   # empty grid axis
    ]
    for method, opts, kw in bad:
        with pytest.raises(semb.SembError) as e:
            semb.Plan(semb.params(method, **opts, **kw))
        assert e.value.code == semb.E_ARG, (opts, kw)
