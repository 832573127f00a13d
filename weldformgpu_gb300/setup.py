"""Host domain set-up: the reference's particle generators and zone
assignment (src/Domain.cpp), implemented in the C++ library (csrc/wf_setup.cpp)."""
import ctypes as C

import numpy as np

from .domain import lib

_bound = False


def _L():
    global _bound
    L = lib()
    if not _bound:
        L.wf_gen_cylinder.restype = C.c_int64
        L.wf_gen_cylinder.argtypes = [C.c_double] * 7 + [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.wf_gen_box.restype = C.c_int64
        L.wf_gen_box.argtypes = [C.c_double] * 8 + [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.wf_gen_cylinder_lattice.restype = C.c_int64
        L.wf_gen_cylinder_lattice.argtypes = [C.c_double] * 4 + [C.c_uint64, C.POINTER(C.c_double)]
        L.wf_assign_zone.restype = C.c_int64
        L.wf_assign_zone.argtypes = [C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_uint8)]
        _bound = True
    return L


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def gen_cylinder_ref(start, R, L, r, density):
    """Domain::AddCylinderLength (src/Domain.cpp:490-573): (x[n,3], mass)."""
    lib_ = _L()
    m = C.c_double()
    n = lib_.wf_gen_cylinder(start[0], start[1], start[2], R, L, r, density, None, C.byref(m))
    x = np.empty(3 * n, dtype=np.float64)
    lib_.wf_gen_cylinder(start[0], start[1], start[2], R, L, r, density, _p(x), C.byref(m))
    return x.reshape(n, 3), m.value


def gen_box_cubic(start, dims, r, density):
    """Domain::AddBoxLength, cubic packing (src/Domain.cpp:296-338): (x[n,3], mass)."""
    lib_ = _L()
    m = C.c_double()
    args = [float(v) for v in list(start) + list(dims)] + [r, density]
    n = lib_.wf_gen_box(*args, None, C.byref(m))
    x = np.empty(3 * n, dtype=np.float64)
    lib_.wf_gen_box(*args, _p(x), C.byref(m))
    return x.reshape(n, 3), m.value


def gen_cylinder_uniform(Rxy, Lz, r, density, ang=2.0 * np.pi, rows=1, r_i=0.0, tag=0):
    """Domain::AddCylUniformLength (src/Domain.cpp:1071-1192): (x[n,3], ids[n], mass)."""
    lib_ = _L()
    fn = lib_.wf_gen_cylinder_uniform
    fn.restype = C.c_int64
    fn.argtypes = [C.c_double] * 5 + [C.c_int, C.c_double, C.c_int32, C.POINTER(C.c_double),
                                      C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    m = C.c_double()
    n = fn(Rxy, Lz, r, density, ang, rows, r_i, tag, None, None, C.byref(m))
    x = np.empty(3 * n)
    ids = np.empty(n, np.int32)
    fn(Rxy, Lz, r, density, ang, rows, r_i, tag, _p(x), _p(ids, C.c_int32), C.byref(m))
    return x.reshape(n, 3), ids, m.value


def gen_icosphere(R, center, level, lower_half=True):
    """Icosphere tool (outward normals): (nodes[nn,3], tris[ne,3])."""
    lib_ = _L()
    fn = lib_.wf_gen_icosphere
    fn.restype = C.c_int64
    fn.argtypes = [C.c_double, C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_double),
                   C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    c = np.asarray(center, dtype=np.float64)
    nn = C.c_int64()
    ne = fn(R, _p(c), int(level), int(lower_half), None, None, C.byref(nn))
    nodes = np.empty(3 * nn.value)
    tris = np.empty(3 * ne, np.int32)
    fn(R, _p(c), int(level), int(lower_half), _p(nodes), _p(tris, C.c_int32), C.byref(nn))
    return nodes.reshape(-1, 3), tris.reshape(-1, 3)


def gen_cylinder_lattice(R, H, dx, jitter, seed):
    """Jittered cubic lattice inside a cylinder (the compression benchmarks' workload)."""
    lib_ = _L()
    n = lib_.wf_gen_cylinder_lattice(R, H, dx, jitter, seed, None)
    x = np.empty(3 * n, dtype=np.float64)
    lib_.wf_gen_cylinder_lattice(R, H, dx, jitter, seed, _p(x))
    return x.reshape(n, 3)


def gen_plane_mesh(axis, positive, p1, p2, dens):
    """TriMesh_d::AxisPlaneMesh (src/cuda/Mesh.cu:48-194): (nodes[nn,3], tris[ne,3], normals[ne,3])."""
    lib_ = _L()
    a, b = np.asarray(p1, dtype=np.float64), np.asarray(p2, dtype=np.float64)
    ne = lib_.wf_gen_plane_mesh(int(axis), int(positive), _p(a), _p(b), int(dens), None, None, None)
    if ne < 0:
        raise ValueError("bad plane mesh arguments")
    nodes = np.empty(3 * (dens + 1) ** 2, dtype=np.float64)
    tris = np.empty(3 * ne, dtype=np.int32)
    normals = np.empty(3 * ne, dtype=np.float64)
    lib_.wf_gen_plane_mesh(int(axis), int(positive), _p(a), _p(b), int(dens), _p(nodes),
                           _p(tris, C.c_int32), _p(normals))
    return nodes.reshape(-1, 3), tris.reshape(-1, 3), normals.reshape(-1, 3)


def assign_zone(x, start, end, zone, ids, not_write):
    """Domain::AssignZone (src/Domain.cpp:989-1005); modifies ids / not_write in place."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    s = np.asarray(start, dtype=np.float64)
    e = np.asarray(end, dtype=np.float64)
    return _L().wf_assign_zone(_p(x), len(x), _p(s), _p(e), int(zone), _p(ids, C.c_int32),
                               _p(not_write, C.c_uint8))
