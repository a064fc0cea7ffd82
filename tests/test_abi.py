"""The C ABI: the library loads, exports every symbol include/cryoim.h declares, and its
host-only entry points (parameters, error codes) behave like the reference's set-up
(0initialvalue.f90, 0calc_initialvalues.f90).  No GPU needed."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "cryoim.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cryoim_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(built):
    import cryoim_gb300._abi as abi
    lib = C.CDLL(abi.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 28
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers the whole ABI
    assert set(syms) <= set(abi.SIGNATURES), set(syms) - set(abi.SIGNATURES)


def test_params_derivation_matches_reference_arithmetic(built):
    import cryoim_gb300 as ci
    # BASELINE config 1: box 128, 2.0 A/px, band 1/60 - 1/10 A^-1
    p = ci.default_params(128, apix=2.0, minRes=60.0, maxRes=10.0, searchstep=1.0)
    assert (p.min_r, p.max_r) == (4, 26)  # 25.6 -> 25 -> forced even 26
    assert p.imgmask_px == np.float32(62.0) / np.float32(2.0)  # default (N/2-2) divided by apix
    f = np.float32
    maxres = f(f(2.0) * f(128)) / f(10.0)
    assert p.delta_angle == f(f(360.0) / f(f(maxres * np.sqrt(f(5.0))) * f(3.14159)))
    # config 2: box 256, 1.5 A/px, band 1/50 - 1/6
    p = ci.default_params(256, apix=1.5, minRes=50.0, maxRes=6.0)
    assert (p.min_r, p.max_r) == (7, 64)
    # code defaults that differ from the help text (0input_parameters.f90:40-51)
    assert p.subrec == 0 and p.maxcentshift == 100.0 and p.ncycle == 6 and p.searchstep == 2.0
    assert p.vol == 300.0 and p.cs == np.float32(2.7) and p.ampwg == np.float32(0.1)


def test_error_codes_without_device(built):
    import cryoim_gb300._abi as abi
    lib = abi.load()
    assert lib.cryoim_params_default(None, 128) == abi.ERR_ARG
    p = abi.Params()
    assert lib.cryoim_params_default(C.byref(p), 7) == abi.ERR_SIZE
    assert lib.cryoim_params_default(C.byref(p), 64) == 0
    p.apix = 0.0
    assert lib.cryoim_params_derive(C.byref(p)) == abi.ERR_ARG
    assert b"positive" in lib.cryoim_last_error()
    assert lib.cryoim_set_params(None, C.byref(p)) == abi.ERR_ARG
    assert lib.cryoim_globesearch(None, None, None, 0, None) == abi.ERR_ARG
    assert lib.cryoim_transform_ort(4, None, None, None, 0) == abi.ERR_ARG
    if not gpu_available():
        h = C.c_void_p()
        assert lib.cryoim_ctx_create(0, C.byref(h)) in (abi.ERR_CUDA, abi.ERR_ARG)
        assert not h.value


def test_no_cpu_fallback_when_library_missing(tmp_path):
    import cryoim_gb300._abi as abi
    with pytest.raises(ImportError):
        abi.load(str(tmp_path / "absent.so"))


def test_oracle_params_and_records_match_the_library(built, orc):
    """The oracle's restatement of the parameter set-up and its record layouts agree
    with the library byte for byte, so either side's records pass to the other."""
    import cryoim_gb300 as ci
    for n, kw in [(256, dict(apix=1.5, minRes=50.0, maxRes=6.0, searchstep=1.0, ampwg=0.07, imgmask=189.0)),
                  (128, dict(apix=2.0, minRes=60.0, maxRes=10.0)), (96, dict(apix=3.0, use_imgmask=0)),
                  (64, {})]:
        a, b = orc.default_params(n, **kw), ci.default_params(n, **kw)
        assert C.sizeof(a) == C.sizeof(b)
        assert C.string_at(C.addressof(a), C.sizeof(a)) == C.string_at(C.addressof(b), C.sizeof(b)), (n, kw)
    assert orc.PARTICLE_DTYPE == ci.PARTICLE_DTYPE and orc.TEMPLATE_DTYPE == ci.TEMPLATE_DTYPE
