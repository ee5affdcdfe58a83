"""The C ABI library loads and exports every function include/pf_cuda.h
declares; host-side parameter handling mirrors Profile::parameter. No GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^PF_API\s+[\w\s\*]*?\b(pf_\w+)\s*\(", text, flags=re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build_cuda()
    from libprofit_gb300 import _ffi
    return _ffi.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_binding_covers_header():
    from libprofit_gb300 import _ffi
    assert declared_symbols() == set(_ffi.exported_symbols())


def test_struct_layout_matches_header():
    from libprofit_gb300 import _ffi
    # pf_profile_desc: 5 int32 + 2 uint32 (28 B, padded to 32) + 3 + 12 doubles
    assert ctypes.sizeof(_ffi.ProfileDesc) == 32 + 15 * 8
    assert ctypes.sizeof(_ffi.ModelDesc) == 112


def test_version_and_errors_without_gpu(lib):
    assert b"sm_103a" in lib.pf_version()
    import libprofit_gb300 as pg
    m = pg.Model(0, 10)
    m.add_profile("sersic")
    with pytest.raises(pg.InvalidParameter, match="dimensions are 0"):
        m.output_dims()
    m = pg.Model(10, 10)
    p = m.add_profile("sersic")
    p.parameter("convolve", True)
    with pytest.raises(pg.InvalidParameter, match="No psf provided"):
        m.output_dims()


def test_parameter_registry():
    import libprofit_gb300 as pg
    p = pg.Profile("sersic")
    p.parameter("re", 3.5)
    p.parameter("nser=2.5")
    p.parameter("rough", True)
    p.parameter("max_recursions", 4)
    assert p.get("re") == 3.5 and p.get("nser") == 2.5 and p.get("rough") == 1
    assert p.get("max_recursions") == 4
    with pytest.raises(pg.InvalidParameter, match="Unknown double parameter in profile sersic: fwhm"):
        p.parameter("fwhm", 1.0)
    with pytest.raises(pg.UnknownParameter):
        p.parameter("fwhm=1")
    with pytest.raises(pg.InvalidParameter, match="missing ="):
        p.parameter("re")
    with pytest.raises(pg.InvalidParameter, match="Unknown profile name"):
        pg.Profile("gaussian")
    assert pg.Profile("ferrer").desc.acc == 1.0
    assert pg.Profile("ferrers").kind == "ferrer"
