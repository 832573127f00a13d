"""The C ABI library: loads, exports every entry point the header declares,
and fails loudly (no CPU fallback) where no GPU is present."""
import ctypes
import os
import re

import numpy as np
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
    sl = tmp_path / "slice.json"        # main's default sliceAngle (2.0000001 pi): a slice
    sl.write_text(amp.read_text().replace('"Box"', '"Cylinder", "gridCoordSys": "Cylindrical"'))
    assert L.wf_run_json(str(sl).encode(), None, err, 512) == -1
    assert b"axisymmetric" in err.value
    if not has_gpu:   # a complete input is parsed, then the domain needs the GPU
        good = tmp_path / "good.json"
        good.write_text(amp.read_text().replace('"valueType": 1', '"valueType": 0'))
        assert L.wf_run_json(str(good).encode(), str(tmp_path).encode(), err, 512) == -2


def _nastran_deck(path):
    """A fixed-field (8-character) deck: GRID id, cp, x, y, z with implicit
    exponents, and CTRIA3 eid, pid, g1, g2, g3 referring to node ids."""
    # negative values fill the 8 characters, as mesh generators write them; a
    # right-justified "    -4.0" reads as 0 in the reference's parser (its
    # first '-' is not the field's first character, so it is taken for an
    # exponent sign) and here alike
    coords = [("0.0", "0.0", "0.0"), ("1.25-03", "0.0", "0.0"), ("0.0", "-2.500-3", "0.5+2"),
              ("-.750000", "3.0", "-1.0+1"), ("2.0-1", "-4.00000", "7.125"),
              ("0.0", "-4.0", "1.0")]
    expect = [(0.0, 0.0, 0.0), (1.25e-3, 0.0, 0.0), (0.0, -2.5e-3, 50.0),
              (-0.75, 3.0, -10.0), (0.2, -4.0, 7.125), (0.0, 0.0, 1.0)]
    ids = [11, 12, 20, 31, 40, 41]
    lines = ["$ deck written by the test", "BEGIN BULK"]
    for i, (x, y, z) in zip(ids, coords):
        lines.append("GRID    %8d%8d%8s%8s%8s" % (i, 0, x, y, z))
    tris = [(11, 12, 20), (12, 31, 20), (31, 40, 20)]
    for e, (a, b, c) in enumerate(tris):
        lines.append("CTRIA3  %8d%8d%8d%8d%8d" % (e + 1, 1, a, b, c))
    lines.append("ENDDATA")
    path.write_text("\n".join(lines) + "\n")
    pos = {i: k for k, i in enumerate(ids)}
    return np.array(expect), np.array([[pos[a], pos[b], pos[c]] for a, b, c in tris], np.int32)


def _read_nastran(fn, path):
    n = ctypes.c_int64()
    ne = fn(str(path).encode(), None, None, ctypes.byref(n))
    assert ne > 0
    nodes = np.empty(3 * n.value)
    tris = np.empty(3 * ne, np.int32)
    fn(str(path).encode(), nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
       tris.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(n))
    return nodes.reshape(-1, 3), tris.reshape(-1, 3)


def _bind_reader(L, name):
    fn = getattr(L, name)
    fn.restype = ctypes.c_int64
    fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)]
    return fn


def test_nastran_reader_implicit_exponents_and_reference_parser(tmp_path):
    from weldformgpu_gb300.domain import lib
    from oracle import oracle as O
    rd = _bind_reader(lib(), "wf_read_nastran")
    deck = tmp_path / "tool.nas"
    expect, etris = _nastran_deck(deck)
    nodes, tris = _read_nastran(rd, deck)
    assert np.array_equal(nodes, expect) and np.array_equal(tris, etris)
    assert rd(str(tmp_path / "none.nas").encode(), None, None, None) == -6
    ref = O.ref_lib()
    if ref is None:
        pytest.skip("reference tree absent: reference parser not built")
    rr = _bind_reader(ref, "wfr_read_nastran")
    import contextlib
    import io
    with contextlib.redirect_stdout(io.StringIO()):
        rn, rt = _read_nastran(rr, deck)
    assert np.array_equal(rn, nodes) and np.array_equal(rt, tris)
    from oracle import build_ref
    example = os.path.join(build_ref.reference_dir(), "examples", "input", "tool_metal_cut_mm.nas")
    if os.path.exists(example):
        a = _read_nastran(rd, example)
        b = _read_nastran(rr, example)
        assert all(np.array_equal(x, y) for x, y in zip(a, b)) and len(a[1]) == 1388


def test_header_documents_reference_citations():
    text = open(HEADER).read()
    # each reference-facing setter cites the Domain_d member it replaces
    for name in ("Set_h", "SetDensity", "SetShearModulus", "SetSigmay", "SetCs", "SetFreePart",
                 "SetID", "MechFraserSolve", "ThermalSolve", "WriteCSV"):
        assert name in text, name


def _lsdyna_deck(path):
    """An LS-DYNA keyword deck: *NODE in fixed fields (8, 16, 16, 16) and in
    free format, *ELEMENT_SPH (fields 8, 8, 16; one free-format card), two node
    sets (the second, titled, overrides the first for a shared node), comments,
    keywords the reader skips, a node that no SPH element uses."""
    lines = ["*KEYWORD", "$ SPH particles written by the test", "*NODE",
             "$    nid               x               y               z",
             "%8d%16s%16s%16s" % (7, "0.0", "0.0", "0.0"),
             "%8d%16s%16s%16s" % (9, "1.0e-3", "-2.5E-4", "0.125"),
             "12, 2.0e-3, 0.0, 1.0e-3",
             "%8d%16s%16s%16s" % (15, "-1.5", "3.0", "4.0"),
             "%8d%16s%16s%16s" % (99, "9.0", "9.0", "9.0"),
             "*PART", "this card is skipped", "         1         1",
             "*ELEMENT_SPH",
             "$    nid     pid            mass",
             "%8d%8d%16s" % (9, 1, "2.5e-6"),
             "%8d%8d%16s" % (7, 1, "1.0e-6"),
             "15, 1, 4.0e-6",
             "%8d%8d%16s" % (12, 1, "3.0e-6"),
             "*SET_NODE_LIST",
             "%10d%10s%10s%10s%10s" % (2, "0.0", "0.0", "0.0", "0.0"),
             "%10d%10d" % (7, 12),
             "*SET_NODE_LIST_TITLE",
             "top platen",
             "%10d" % 3,
             "%10d%10d%10d" % (12, 15, 99),
             "*END"]
    path.write_text("\n".join(lines) + "\n")
    x = np.array([[1.0e-3, -2.5e-4, 0.125], [0.0, 0.0, 0.0], [-1.5, 3.0, 4.0], [2.0e-3, 0.0, 1.0e-3]])
    m = np.array([2.5e-6, 1.0e-6, 4.0e-6, 3.0e-6])
    ids = np.array([0, 2, 3, 3], np.int32)
    return x, m, ids


def test_lsdyna_reader_known_answer(tmp_path):
    from weldformgpu_gb300.domain import lib
    L = lib()
    fn = L.wf_read_lsdyna
    fn.restype = ctypes.c_int64
    fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)]
    deck = tmp_path / "particles.k"
    ex, em, eid = _lsdyna_deck(deck)
    n = fn(str(deck).encode(), None, None, None)
    assert n == 4
    x = np.empty(3 * n)
    m = np.empty(n)
    ids = np.empty(n, np.int32)
    assert fn(str(deck).encode(), x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              m.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) == 4
    assert np.array_equal(x.reshape(-1, 3), ex) and np.array_equal(m, em)
    assert np.array_equal(ids, eid)
    assert fn(str(tmp_path / "none.k").encode(), None, None, None) == -6
    bad = tmp_path / "bad.k"
    bad.write_text("*NODE\n       1             0.0             0.0             0.0\n"
                   "*ELEMENT_SPH\n       5       1          1.0e-6\n")
    assert fn(str(bad).encode(), None, None, None) == -1        # element on an unknown node
    empty = tmp_path / "empty.k"
    empty.write_text("*NODE\n       1             0.0             0.0             0.0\n")
    assert fn(str(empty).encode(), None, None, None) == -1      # no SPH element


def test_header_compiles_as_c99_and_cpp():
    """The boundary is a C ABI: the header alone compiles as C99 and as C++
    (what a cgo, JNI or plain C caller would include)."""
    import shutil
    import subprocess
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                       "weldform_gb300.h")
    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if gcc is None or gxx is None:
        pytest.skip("no host compiler")
    for cmd in ([gcc, "-fsyntax-only", "-x", "c", "-std=c99", "-Wall", "-Werror", hdr],
                [gxx, "-fsyntax-only", "-x", "c++", "-Wall", "-Werror", hdr]):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, (cmd, r.stderr)
