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


def test_json_driver_rejects_bad_inputs_before_any_gpu_work(tmp_path, has_gpu):
    from weldformgpu_gb300.domain import lib
    L = lib()
    L.wf_run_json.restype = ctypes.c_int
    L.wf_run_json.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64]
    err = ctypes.create_string_buffer(512)
    assert L.wf_run_json(str(tmp_path / "missing.json").encode(), None, err, 512) == -6
    bad = tmp_path / "bad.json"
    bad.write_text('{"Configuration": {"particleRadius": 0.001,, }')
    assert L.wf_run_json(str(bad).encode(), None, err, 512) == -6
    assert b"syntax" in err.value
    nocfg = tmp_path / "nocfg.json"
    nocfg.write_text('{"Materials": [{"type": "Bilinear"}]}')
    assert L.wf_run_json(str(nocfg).encode(), None, err, 512) == -1
    assert b"particleRadius" in err.value
    amp = tmp_path / "amp.json"
    amp.write_text('{"Configuration": {"particleRadius": 0.001, "hFactor": 1.2, "simTime": 1e-6,'
                   ' "outTime": 1e-7}, "Materials": [{"type": "Bilinear", "const": [7e8],'
                   ' "density0": 2700, "youngsModulus": 7e10, "poissonsRatio": 0.3,'
                   ' "yieldStress0": 3e8}], "DomainBlocks": [{"type": "Box", "start": [0, 0, 0],'
                   ' "dim": [0.01, 0.01, 0.01]}], "BoundaryConditions": [{"zoneId": 1,'
                   ' "valueType": 1}]}')
    assert L.wf_run_json(str(amp).encode(), None, err, 512) == -1
    assert b"amplitude" in err.value
    if not has_gpu:   # a complete input is parsed, then the domain needs the GPU
        good = tmp_path / "good.json"
        good.write_text(amp.read_text().replace('"valueType": 1', '"valueType": 0'))
        assert L.wf_run_json(str(good).encode(), str(tmp_path).encode(), err, 512) == -2


def test_header_documents_reference_citations():
    text = open(HEADER).read()
    # each reference-facing setter cites the Domain_d member it replaces
    for name in ("Set_h", "SetDensity", "SetShearModulus", "SetSigmay", "SetCs", "SetFreePart",
                 "SetID", "MechFraserSolve", "ThermalSolve", "WriteCSV"):
        assert name in text, name
