"""The reference's input-file driver (wf_run_json and the `wf` executable).

An input file in the reference's format (the keys of src/WeldFormGPU.cu's
main) runs end to end; its CSV snapshots have the reference's columns and
its final state equals the same set-up built through the Python API.
"""
import ctypes
import json
import math
import os
import subprocess

import numpy as np
import pytest

from weldformgpu_gb300 import _abi
from weldformgpu_gb300 import setup as P

pytestmark = pytest.mark.gpu

HEADER = ("ID, X, Y, Z, posX,posY,posZ,Ux, Uy, Uz, Vx, Vy, Vz, Ax, Ay, Az, rho, p, SigmaEq, "
          "Pl_Strain, Nb, ContNb, CFx, CFy, CFz, Nx, Ny, Nz, h")

R, H, r = 0.0025, 0.005, 0.00025
E, nu, rho, Fy, Et = 70e9, 0.33, 2700.0, 300e6, 7e8
SIM, OUT = 2.0e-5, 5.0e-6


def _inputs():
    x, _ = P.gen_cylinder_ref((0.0, 0.0, 0.0), R, H, r, rho)
    h = 1.2 * 2 * r
    zp = float(x[:, 2].max()) + h + 1e-7
    cfg = {
        "Configuration": {"particleRadius": r, "hFactor": 1.2, "simTime": SIM, "outTime": OUT},
        "Materials": [{"id": "Solid", "type": "Bilinear", "const": [Et], "density0": rho,
                       "youngsModulus": E, "poissonsRatio": nu, "yieldStress0": Fy}],
        "DomainBlocks": [{"type": "Cylinder", "zoneId": 0, "start": [0.0, 0.0, 0.0],
                          "dim": [2 * R, 0.0, H]}],
        "DomainZones": [{"id": 2, "start": [-1.0, -1.0, -1.0], "end": [1.0, 1.0, 0.0004]}],
        "RigidBodies": [{"type": "Plane", "zoneId": 10, "start": [-0.003, -0.003, zp],
                         "partSide": 6, "dim": [0.006, 0.006, 0.0]}],
        "Contact": [{"fricCoeffStatic": 0.3, "fricCoeffDynamic": 0.2}],
        "BoundaryConditions": [{"zoneId": 2, "value": [0.0, 0.0, 0.0], "free": True},
                               {"zoneId": 10, "valuetype": 0, "value": [0.0, 0.0, -10.0],
                                "free": True}],
    }
    return cfg, zp


def _api_domain(zp, mesh=None, law=0):
    """main's set-up (src/WeldFormGPU.cu:689-914) through the Python API;
    mesh = (nodes, tris) of a file rigid body, else main's plane; law 1 with
    contact_dx = 2 r as the driver's "law" key sets it."""
    from weldformgpu_gb300 import Domain_d
    x, mass = P.gen_cylinder_ref((0.0, 0.0, 0.0), R, H, r, rho)
    ns = len(x)
    ids = np.zeros(ns, np.int32)
    P.assign_zone(x, (-1, -1, -1), (1, 1, 0.0004), 2, ids, np.zeros(ns, np.uint8))
    if mesh is None:
        nodes, tris, normals = P.gen_plane_mesh(2, 0, (-0.003, -0.003, zp), (0.003, 0.003, zp), 6)
    else:
        (nodes, tris), normals = mesh, None
    n = ns + len(tris)
    K, G = E / (3 * (1 - 2 * nu)), E / (2 * (1 + nu))
    Cs, h = math.sqrt(K / rho), 1.2 * 2 * r
    d = Domain_d(n)
    d.set_solid_count(ns)
    d.set_material(_abi.WfMaterial(model=_abi.WF_BILINEAR, E=E, nu=nu, sy0=Fy, Et=Et))
    d.set_density(rho)
    d.set_h(h)
    d.set_positions(np.vstack([x, np.zeros((len(tris), 3))]))
    d.set_mass(np.concatenate([np.full(ns, mass), np.zeros(len(tris))]))
    d.set_shear_modulus(G)
    d.set_free(np.ones(n, np.uint8))
    d.set_id(np.concatenate([ids, np.full(len(tris), 10, np.int32)]))
    d.set_cs(np.full(n, Cs))
    d.set_sigma_y(Fy)
    d.set_not_write_surf_id(np.concatenate([(ids != 0).astype(np.uint8), np.zeros(len(tris), np.uint8)]))
    d.set_temperature(np.full(n, 20.0))
    d.set_time_step(0.4 * h / (Cs + 10.0))
    d.add_velocity_bc(2, 0.0, 0.0, 0.0)
    d.add_velocity_bc(10, 0.0, 0.0, -10.0)
    d.add_trimesh(nodes, tris, 10, ns, (0.0, 0.0, -10.0), normals=normals)
    d.set_contact(0.3, 0.2, law)
    if law == 1:
        d.set_option("contact_dx", 2 * r)
    d.mech_fraser_solve(SIM, OUT)
    return d, n


def _csv(path):
    with open(path) as f:
        head = f.readline().strip()
        rows = np.loadtxt(f, delimiter=",")
    return head, rows


def test_json_driver_matches_api_and_writes_reference_csv(tmp_path):
    from weldformgpu_gb300.domain import LIB_PATH, lib
    lib()
    L = ctypes.CDLL(LIB_PATH)
    L.wf_run_json.restype = ctypes.c_int
    L.wf_run_json.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64]
    cfg, zp = _inputs()
    inp = tmp_path / "Contact_Compression_small.json"
    inp.write_text(json.dumps(cfg, indent=1))
    out = tmp_path / "run"
    out.mkdir()
    err = ctypes.create_string_buffer(512)
    assert L.wf_run_json(str(inp).encode(), str(out).encode(), err, 512) == 0, err.value
    snaps = sorted(f for f in os.listdir(out) if f.startswith("out_"))
    assert snaps[0] == "out_0.000000.csv" and len(snaps) >= int(SIM / OUT)
    head, rows = _csv(out / "test.csv")
    assert head == HEADER
    d, n = _api_domain(zp)
    assert rows.shape == (n, 29)
    np.testing.assert_allclose(rows[:, 1:4], d.get_field("x"), rtol=2e-6, atol=1e-12)
    np.testing.assert_allclose(rows[:, 19], d.get_field("pl_strain"), rtol=2e-6, atol=1e-12)
    assert np.array_equal(rows[:, 0].astype(np.int32), d.get_field_i32("ID"))
    assert (rows[:, 21] > 0).sum() > 20                       # contact neighbours written
    assert np.abs(rows[:, 22:25]).sum() > 0                   # contact forces written
    # the command-line executable gives the same file
    exe = os.path.join(os.path.dirname(LIB_PATH), "wf")
    out2 = tmp_path / "cli"
    out2.mkdir()
    subprocess.run([exe, str(inp), str(out2)], check=True, capture_output=True)
    assert (out2 / "test.csv").read_bytes() == (out / "test.csv").read_bytes()


def test_json_driver_cylindrical_grid(tmp_path):
    """DomainBlocks Cylinder on the "Cylindrical" grid (AddCylUniformLength)
    with sliceAngle 2 pi: the particle set of the generator, axis ids kept."""
    from weldformgpu_gb300.domain import LIB_PATH, lib
    lib()
    L = ctypes.CDLL(LIB_PATH)
    L.wf_run_json.restype = ctypes.c_int
    L.wf_run_json.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64]
    cfg, _ = _inputs()
    cfg.pop("RigidBodies")
    cfg.pop("Contact")
    cfg["DomainBlocks"] = [{"type": "Cylinder", "gridCoordSys": "Cylindrical",
                            "sliceAngle": 2.0 * math.pi, "start": [0.0, 0.0, 0.0],
                            "dim": [2 * R, 0.0, H]}]
    cfg["BoundaryConditions"] = [{"zoneId": 2, "value": [0.0, 0.0, 0.0]}]
    cfg["Configuration"]["simTime"] = 2.0e-6
    inp = tmp_path / "cyl.json"
    inp.write_text(json.dumps(cfg))
    err = ctypes.create_string_buffer(512)
    assert L.wf_run_json(str(inp).encode(), str(tmp_path).encode(), err, 512) == 0, err.value
    x, ids, _ = P.gen_cylinder_uniform(R, H, r, rho)
    head, rows = _csv(tmp_path / "test.csv")
    assert rows.shape[0] == len(x)
    got = rows[:, 0].astype(np.int32)
    # axis particles keep id 4 unless the bottom zone (z <= 0.4 mm) takes them
    assert (got == 4).sum() == ((ids == 4) & (x[:, 2] > 0.0004)).sum() > 0
    assert (got == 2).sum() > 0                                  # the bottom zone


def test_json_driver_nastran_rigid_body(tmp_path):
    """RigidBodies type "File": a plane tool written as a fixed-field Nastran
    deck (normal -z from its node order) gives the run the API gives with the
    mesh read by wf_read_nastran."""
    from weldformgpu_gb300.domain import LIB_PATH, lib
    lib()
    L = ctypes.CDLL(LIB_PATH)
    L.wf_run_json.restype = ctypes.c_int
    L.wf_run_json.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64]
    L.wf_read_nastran.restype = ctypes.c_int64
    L.wf_read_nastran.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)]
    cfg, zp = _inputs()
    # an 8-character field that is not below zp: mantissa and implicit exponent
    zs = "%.4f-3" % (math.ceil(zp * 1e7) / 1e4)
    grid = [-0.003, -0.002, -0.001, 0.0, 0.001, 0.002, 0.003]
    lines = ["$ plane tool", "BEGIN BULK"]
    for j, y in enumerate(grid):
        for i, x in enumerate(grid):
            lines.append("GRID    %8d%8d%8s%8s%8s" % (1 + 7 * j + i, 0, "%.5f" % x, "%.5f" % y, zs))
    e = 1
    for j in range(6):
        for i in range(6):
            a, b = 1 + 7 * j + i, 2 + 7 * j + i
            c, d = a + 7, b + 7
            for t in ((a, c, b), (b, c, d)):               # normal -z
                lines.append("CTRIA3  %8d%8d%8d%8d%8d" % (e, 1, *t))
                e += 1
    deck = tmp_path / "tool.nas"
    deck.write_text("\n".join(lines) + "\n")
    cfg["RigidBodies"] = [{"type": "File", "zoneId": 10, "fileName": "tool.nas"}]
    inp = tmp_path / "file_tool.json"
    inp.write_text(json.dumps(cfg))
    out = tmp_path / "run"
    out.mkdir()
    err = ctypes.create_string_buffer(512)
    assert L.wf_run_json(str(inp).encode(), str(out).encode(), err, 512) == 0, err.value
    nn = ctypes.c_int64()
    ne = L.wf_read_nastran(str(deck).encode(), None, None, ctypes.byref(nn))
    assert ne == 72 and nn.value == 49
    nodes, tris = np.empty(3 * nn.value), np.empty(3 * ne, np.int32)
    L.wf_read_nastran(str(deck).encode(), nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                      tris.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(nn))
    d, n = _api_domain(zp, (nodes.reshape(-1, 3), tris.reshape(-1, 3)))
    head, rows = _csv(out / "test.csv")
    np.testing.assert_allclose(rows[:, 1:4], d.get_field("x"), rtol=2e-6, atol=1e-12)
    assert (rows[:, 21] > 0).sum() > 20                       # in contact with the tool


def test_json_driver_contact_law1(tmp_path):
    """The extension key Contact[0].law = 1 runs the binned nearest-triangle law
    (contact_dx = 2 r) and equals the same set-up through the API."""
    from weldformgpu_gb300.domain import LIB_PATH, lib
    lib()
    L = ctypes.CDLL(LIB_PATH)
    L.wf_run_json.restype = ctypes.c_int
    L.wf_run_json.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64]
    cfg, zp = _inputs()
    cfg["Contact"][0]["law"] = 1
    # law 1 acts within dx/2 = r of the surface: the plate starts just outside
    zp = zp - 1.2 * 2 * r - 1e-7 + r + 1e-6
    cfg["RigidBodies"][0]["start"][2] = zp
    inp = tmp_path / "law1.json"
    inp.write_text(json.dumps(cfg, indent=1))
    out = tmp_path / "run"
    out.mkdir()
    err = ctypes.create_string_buffer(512)
    assert L.wf_run_json(str(inp).encode(), str(out).encode(), err, 512) == 0, err.value
    head, rows = _csv(out / "test.csv")
    d, n = _api_domain(zp, law=1)
    np.testing.assert_allclose(rows[:, 1:4], d.get_field("x"), rtol=2e-6, atol=1e-12)
    np.testing.assert_allclose(rows[:, 19], d.get_field("pl_strain"), rtol=2e-6, atol=1e-12)
    cf = d.get_field("contforce")
    assert (np.abs(cf).sum(axis=1) > 0).sum() > 20             # the plate touches
    np.testing.assert_allclose(rows[:, 22:25], cf, rtol=2e-6, atol=1e-6 * np.abs(cf).max())
    cfg["Contact"][0]["law"] = 2
    inp.write_text(json.dumps(cfg))
    assert L.wf_run_json(str(inp).encode(), str(out).encode(), err, 512) != 0
    assert b"law" in err.value


def test_json_driver_lsdyna_particle_file(tmp_path):
    """DomainBlocks "File" (main's ReadFromLSdyna path, src/WeldFormGPU.cu:378-398):
    the cylinder's particles written as an LS-DYNA keyword deck (*NODE,
    *ELEMENT_SPH with masses, the fixed bottom zone as a *SET_NODE_LIST of id
    2) give the run of the generator-built input, state for state."""
    from weldformgpu_gb300.domain import LIB_PATH, lib
    lib()
    L = ctypes.CDLL(LIB_PATH)
    L.wf_run_json.restype = ctypes.c_int
    L.wf_run_json.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64]
    x, mass = P.gen_cylinder_ref((0.0, 0.0, 0.0), R, H, r, rho)
    ns = len(x)
    ids = np.zeros(ns, np.int32)
    P.assign_zone(x, (-1, -1, -1), (1, 1, 0.0004), 2, ids, np.zeros(ns, np.uint8))
    lines = ["*KEYWORD", "*NODE"]
    lines += ["%d, %.17g, %.17g, %.17g" % (1000 + i, x[i, 0], x[i, 1], x[i, 2]) for i in range(ns)]
    lines.append("*ELEMENT_SPH")
    lines += ["%d, 1, %.17g" % (1000 + i, mass) for i in range(ns)]
    lines += ["*SET_NODE_LIST", "2"]
    zone = [1000 + i for i in range(ns) if ids[i] == 2]
    lines += [", ".join(str(v) for v in zone[k:k + 8]) for k in range(0, len(zone), 8)]
    lines.append("*END")
    (tmp_path / "particles.k").write_text("\n".join(lines) + "\n")
    cfg, zp = _inputs()
    cfg["DomainBlocks"] = [{"type": "File", "fileName": "particles.k"}]
    cfg.pop("DomainZones")
    inp = tmp_path / "from_file.json"
    inp.write_text(json.dumps(cfg, indent=1))
    out = tmp_path / "run"
    out.mkdir()
    err = ctypes.create_string_buffer(512)
    assert L.wf_run_json(str(inp).encode(), str(out).encode(), err, 512) == 0, err.value
    head, rows = _csv(out / "test.csv")
    d, n = _api_domain(zp)
    assert rows.shape == (n, 29)
    np.testing.assert_allclose(rows[:, 1:4], d.get_field("x"), rtol=2e-6, atol=1e-12)
    np.testing.assert_allclose(rows[:, 19], d.get_field("pl_strain"), rtol=2e-6, atol=1e-12)
    assert np.array_equal(rows[:, 0].astype(np.int32), d.get_field_i32("ID"))
