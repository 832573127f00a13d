"""The C ABI library: loads, exports every entry point the header declares,
and fails loudly (no CPU fallback) where no GPU is present."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "weldform_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from weldformgpu_gb300.domain import LIB_PATH, lib
    lib()
    L = ctypes.CDLL(LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 40
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_version_string():
    from weldformgpu_gb300 import version
    assert "sm_103a" in version()


def test_no_gpu_fails_loudly(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    from weldformgpu_gb300 import Domain_d, WeldformError
    with pytest.raises(WeldformError) as e:
        Domain_d(100)
    assert e.value.code == -2


def test_bad_arguments_rejected_without_touching_the_gpu():
    from weldformgpu_gb300.domain import lib
    L = lib()
    h = ctypes.c_void_p()
    assert L.wf_create(ctypes.byref(h), 0) == -1           # WF_ERR_ARG
    assert L.wf_create(None, 10) == -1
    assert L.wf_destroy(None) == 0
    assert L.wf_set_h(None, 1.0) == -1
    assert L.wf_step(None, 1) == -1


def test_header_documents_reference_citations():
    text = open(HEADER).read()
    # each reference-facing setter cites the Domain_d member it replaces
    for name in ("Set_h", "SetDensity", "SetShearModulus", "SetSigmay", "SetCs", "SetFreePart",
                 "SetID", "MechFraserSolve", "ThermalSolve", "WriteCSV"):
        assert name in text, name
