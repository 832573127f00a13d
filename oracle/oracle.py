"""Python binding of the CPU oracle (oracle/liboracle.so) and of the
reference's kernels compiled for the CPU (oracle/_ref/libwfref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline arm.  The product package never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from weldformgpu_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libwfref.so")
NB = _abi.WF_MAX_NEIGHBORS

# -O2 and -ffp-contract=off: IEEE double arithmetic with no fused multiply-add,
# as the reference's --fmad=false build (src/CMakeLists.txt:29).
CFLAGS = ["-std=gnu11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]


def build(force=False):
    """Compiles oracle/wf_oracle.c into oracle/liboracle.so."""
    src = os.path.join(HERE, "wf_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "wf_oracle.h"))):
        return LIB_PATH
    subprocess.run(["gcc"] + CFLAGS + ["-o", LIB_PATH, src, "-lm"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        _abi.bind(L, "wfo_", _abi.SIGNATURES)
        L.wfo_run_stage.restype = C.c_int
        L.wfo_run_stage.argtypes = [C.c_void_p, C.c_char_p]
        L.wfo_set_field.restype = C.c_int
        L.wfo_set_field.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
        L.wfo_set_threads.restype = C.c_int
        L.wfo_grad_kernel.restype = C.c_double
        L.wfo_grad_kernel.argtypes = [C.c_double, C.c_double]
        L.wfo_set_threads.argtypes = [C.c_int]
        L.wfo_set_mlp_params.restype = C.c_int
        L.wfo_set_mlp_params.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        for name in ("wfo_gen_cylinder_ref", "wfo_gen_box_cubic"):
            fn = getattr(L, name)
            fn.restype = C.c_int64
            fn.argtypes = [C.c_double] * 8 + [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.wfo_gen_cylinder_ref.argtypes = [C.c_double] * 7 + [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.wfo_gen_cylinder_lattice.restype = C.c_int64
        L.wfo_gen_cylinder_lattice.argtypes = [C.c_double] * 4 + [C.c_uint64, C.POINTER(C.c_double)]
        L.wfo_assign_zone.restype = C.c_int64
        L.wfo_assign_zone.argtypes = [C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int32),
                                      C.POINTER(C.c_uint8)]
        L.wfo_mlp_forward.restype = C.c_int
        L.wfo_mlp_forward.argtypes = [C.POINTER(C.c_double)] * 2 + [C.c_int64, C.POINTER(C.c_double)]
        L.wfo_mlp_loss_grad.restype = C.c_int
        L.wfo_mlp_loss_grad.argtypes = [C.POINTER(C.c_double)] * 3 + [C.c_int64] + [C.POINTER(C.c_double)] * 2
        _lib = L
    return _lib


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def set_threads(n):
    lib().wfo_set_threads(int(n))


class OracleError(RuntimeError):
    pass


class OracleDomain:
    """Same method names as weldformgpu_gb300.Domain_d, backed by the oracle."""

    def __init__(self, n):
        self.L = lib()
        self.h = C.c_void_p()
        rc = self.L.wfo_create(C.byref(self.h), int(n))
        if rc:
            raise OracleError("wfo_create failed (%d)" % rc)
        self.n = int(n)

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.wfo_destroy(self.h)
            self.h = C.c_void_p()

    def _ck(self, rc, what):
        if rc != 0:
            raise OracleError("%s: %s (%s)" % (what, _abi.ERROR_NAMES.get(rc, rc),
                                               self.L.wfo_last_error(self.h).decode()))

    def __getattr__(self, name):
        # scalar setters / solvers: forwarded with the prefix
        fn = getattr(self.L, "wfo_" + name, None)
        if fn is None:
            raise AttributeError(name)

        def call(*args):
            conv = []
            for a in args:
                if isinstance(a, np.ndarray):
                    if a.dtype == np.float64:
                        conv.append(_p(np.ascontiguousarray(a)))
                    elif a.dtype == np.int32:
                        conv.append(_p(np.ascontiguousarray(a), C.c_int32))
                    elif a.dtype == np.uint8 or a.dtype == np.bool_:
                        conv.append(_p(np.ascontiguousarray(a, dtype=np.uint8), C.c_uint8))
                    else:
                        raise TypeError(a.dtype)
                elif isinstance(a, str):
                    conv.append(a.encode())
                else:
                    conv.append(a)
            self._ck(fn(self.h, *conv), name)
        return call

    def set_material(self, mat):
        self._ck(self.L.wfo_set_material(self.h, C.byref(mat)), "set_material")

    def set_mlp_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        self._ck(self.L.wfo_set_mlp_params(self.h, _p(p)), "set_mlp_params")

    def set_contact(self, mu_static, mu_dynamic, law=0):
        self._ck(self.L.wfo_set_contact(self.h, float(mu_static), float(mu_dynamic), int(law)),
                 "set_contact")

    def add_trimesh(self, nodes, tris, zone_id, first, vel, angvel=(0.0, 0.0, 0.0), normals=None):
        nd = np.ascontiguousarray(nodes, dtype=np.float64).reshape(-1, 3)
        tr = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
        na = None if normals is None else np.ascontiguousarray(normals, dtype=np.float64)
        v = np.ascontiguousarray(vel, dtype=np.float64)
        w = np.ascontiguousarray(angvel, dtype=np.float64)
        self._ck(self.L.wfo_add_trimesh(self.h, _p(nd), len(nd), _p(tr, C.c_int32), len(tr),
                                        None if na is None else _p(na), int(zone_id), int(first),
                                        _p(v), _p(w)), "add_trimesh")

    def get_field(self, name):
        c = _abi.FIELD_COMPONENTS.get(name, 1)
        out = np.empty(self.n * c, dtype=np.float64)
        self._ck(self.L.wfo_get_field(self.h, name.encode(), _p(out)), "get_field " + name)
        return out.reshape(self.n, c) if c > 1 else out

    def set_field(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        self._ck(self.L.wfo_set_field(self.h, name.encode(), _p(a)), "set_field " + name)

    def get_field_i32(self, name):
        out = np.empty(self.n, dtype=np.int32)
        self._ck(self.L.wfo_get_field_i32(self.h, name.encode(), _p(out, C.c_int32)), name)
        return out

    def get_neighbors(self):
        cnt = np.empty(self.n, dtype=np.int32)
        lst = np.empty(self.n * NB, dtype=np.int32)
        self._ck(self.L.wfo_get_neighbors(self.h, _p(cnt, C.c_int32), _p(lst, C.c_int32)),
                 "get_neighbors")
        return cnt, lst.reshape(self.n, NB)

    def get_scalar(self, name):
        out = C.c_double()
        self._ck(self.L.wfo_get_scalar(self.h, name.encode(), C.byref(out)), name)
        return out.value

    def run_stage(self, name):
        self._ck(self.L.wfo_run_stage(self.h, name.encode()), "run_stage " + name)

    def set_velocity_bc(self, index, vx, vy, vz):
        self._ck(self.L.wfo_set_velocity_bc(self.h, int(index), float(vx), float(vy), float(vz)),
                 "set_velocity_bc")

    def get_output_series(self):
        """Output rows (time, step, maxima, contact sums, energy, BC reactions)."""
        n, w = C.c_int64(), C.c_int64()
        self._ck(self.L.wfo_get_output_series(self.h, None, 0, C.byref(n), C.byref(w)),
                 "get_output_series")
        rows = np.empty((n.value, w.value), dtype=np.float64)
        if n.value:
            self._ck(self.L.wfo_get_output_series(self.h, _p(rows), n.value, C.byref(n),
                                                  C.byref(w)), "get_output_series")
        return rows


# ---- generators -----------------------------------------------------------
def gen_cylinder_ref(start, R, L, r, density):
    """Domain::AddCylinderLength; returns (x[n,3], mass)."""
    L_ = lib()
    m = C.c_double()
    n = L_.wfo_gen_cylinder_ref(start[0], start[1], start[2], R, L, r, density, None, C.byref(m))
    x = np.empty(3 * n, dtype=np.float64)
    L_.wfo_gen_cylinder_ref(start[0], start[1], start[2], R, L, r, density, _p(x), C.byref(m))
    return x.reshape(n, 3), m.value


def gen_box_cubic(start, dims, r, density):
    L_ = lib()
    m = C.c_double()
    args = list(start) + list(dims) + [r, density]
    n = L_.wfo_gen_box_cubic(*args, None, C.byref(m))
    x = np.empty(3 * n, dtype=np.float64)
    L_.wfo_gen_box_cubic(*args, _p(x), C.byref(m))
    return x.reshape(n, 3), m.value


def gen_cylinder_uniform(Rxy, Lz, r, density, ang=2.0 * np.pi, rows=1, r_i=0.0, tag=0):
    """AddCylUniformLength restated: (x[n,3], ids[n], mass)."""
    L = lib()
    fn = L.wfo_gen_cylinder_uniform
    fn.restype = C.c_int64
    fn.argtypes = [C.c_double] * 5 + [C.c_int, C.c_double, C.c_int32, C.POINTER(C.c_double),
                                      C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    m = C.c_double()
    n = fn(Rxy, Lz, r, density, ang, rows, r_i, tag, None, None, C.byref(m))
    x = np.empty(3 * n)
    ids = np.empty(n, np.int32)
    fn(Rxy, Lz, r, density, ang, rows, r_i, tag, _p(x), _p(ids, C.c_int32), C.byref(m))
    return x.reshape(n, 3), ids, m.value


def gen_cylinder_lattice(R, H, dx, jitter, seed):
    L_ = lib()
    n = L_.wfo_gen_cylinder_lattice(R, H, dx, jitter, seed, None)
    x = np.empty(3 * n, dtype=np.float64)
    L_.wfo_gen_cylinder_lattice(R, H, dx, jitter, seed, _p(x))
    return x.reshape(n, 3)


def gen_plane_mesh(axis, positive, p1, p2, dens):
    """AxisPlaneMesh restated: (nodes[nn,3], tris[ne,3], normals[ne,3])."""
    L = lib()
    a, b = np.asarray(p1, dtype=np.float64), np.asarray(p2, dtype=np.float64)
    ne = L.wfo_gen_plane_mesh(int(axis), int(positive), _p(a), _p(b), int(dens), None, None, None)
    nodes = np.empty(3 * (dens + 1) ** 2)
    tris = np.empty(3 * ne, dtype=np.int32)
    normals = np.empty(3 * ne)
    L.wfo_gen_plane_mesh(int(axis), int(positive), _p(a), _p(b), int(dens), _p(nodes),
                         _p(tris, C.c_int32), _p(normals))
    return nodes.reshape(-1, 3), tris.reshape(-1, 3), normals.reshape(-1, 3)


def assign_zone(x, start, end, zone, ids, not_write):
    x = np.ascontiguousarray(x, dtype=np.float64)
    s = np.asarray(start, dtype=np.float64)
    e = np.asarray(end, dtype=np.float64)
    return lib().wfo_assign_zone(_p(x), len(x), _p(s), _p(e), int(zone), _p(ids, C.c_int32),
                                 _p(not_write, C.c_uint8))


def mlp_forward(params, xin):
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(xin, dtype=np.float64)
    y = np.empty(len(x), dtype=np.float64)
    rc = lib().wfo_mlp_forward(_p(p), _p(x), len(x), _p(y))
    assert rc == 0
    return y


def mlp_loss_grad(params, xin, target):
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(xin, dtype=np.float64)
    t = np.ascontiguousarray(target, dtype=np.float64)
    g = np.empty_like(p)
    loss = C.c_double()
    rc = lib().wfo_mlp_loss_grad(_p(p), _p(x), _p(t), len(x), C.byref(loss), _p(g))
    assert rc == 0
    return loss.value, g


# ---- the reference compiled for the CPU -------------------------------------
_ref = None


def ref_lib():
    """oracle/_ref/libwfref.so, or None when it was not built (no reference tree)."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        L = C.CDLL(REF_PATH)
        L.wfr_neighbors.restype = C.c_int
        L.wfr_neighbors.argtypes = [C.POINTER(C.c_double), C.c_int64, C.c_double,
                                    C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.wfr_create.restype = C.c_void_p
        L.wfr_create.argtypes = [C.c_int64]
        L.wfr_destroy.argtypes = [C.c_void_p]
        L.wfr_set_scalars.argtypes = [C.c_void_p] + [C.c_double] * 8
        L.wfr_set_material.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 11
        L.wfr_set_arrays.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.wfr_add_bc.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double]
        L.wfr_set_rebuild_every.argtypes = [C.c_void_p, C.c_int]
        L.wfr_begin.argtypes = [C.c_void_p]
        L.wfr_step.argtypes = [C.c_void_p, C.c_int64]
        L.wfr_get.restype = C.c_int
        L.wfr_get.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
        L.wfr_set_hollomon.argtypes = [C.c_void_p] + [C.c_double] * 5
        L.wfr_get_id.restype = C.c_int
        L.wfr_get_id.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.wfr_set_not_write.argtypes = [C.c_void_p, C.POINTER(C.c_uint8)]
        L.wfr_set_contact.argtypes = [C.c_void_p, C.c_double, C.c_double]
        pd = C.POINTER(C.c_double)
        L.wfr_add_trimesh.argtypes = [C.c_void_p, pd, C.c_int, C.POINTER(C.c_int32), C.c_int, pd,
                                      C.c_int, C.c_int64, pd, pd]
        L.wfr_thermal_solve.argtypes = [C.c_void_p, C.c_int64, pd, pd, C.POINTER(C.c_int32),
                                        C.c_double, C.c_double]
        _ref = L
    return _ref


def ref_neighbors(x, h):
    L = ref_lib()
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = len(x)
    cnt = np.empty(n, dtype=np.int32)
    lst = np.empty(n * NB, dtype=np.int32)
    L.wfr_neighbors(_p(x), n, h, _p(cnt, C.c_int32), _p(lst, C.c_int32))
    return cnt, lst.reshape(n, NB)


class RefDomain:
    """The reference's Domain_d kernels, run on the CPU in Fraser-loop order."""

    def __init__(self, n):
        self.L = ref_lib()
        self.h = self.L.wfr_create(int(n))
        self.n = int(n)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.wfr_destroy(self.h)
            self.h = None

    def setup(self, x, m, ids, h, rho, G, sy, Cs, dt, alpha, beta, mat, T=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        m = np.ascontiguousarray(m, dtype=np.float64)
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        Tp = None if T is None else _p(np.ascontiguousarray(T, dtype=np.float64))
        self.L.wfr_set_scalars(self.h, h, rho, G, sy, Cs, dt, alpha, beta)
        if mat.model == _abi.WF_HOLLOMON:
            self.L.wfr_set_hollomon(self.h, mat.E, mat.nu, mat.sy0, mat.K_hol, mat.m_hol)
        else:
            self.L.wfr_set_material(self.h, mat.model, mat.E, mat.nu, mat.Et, mat.A, mat.B, mat.n,
                                    mat.C, mat.eps0, mat.m, mat.Tm, mat.Tt)
        self.L.wfr_set_arrays(self.h, _p(x), _p(m), _p(ids, C.c_int32), Tp)

    def add_bc(self, zone, v):
        self.L.wfr_add_bc(self.h, int(zone), float(v[0]), float(v[1]), float(v[2]))

    def set_not_write(self, flags):
        f = np.ascontiguousarray(flags, dtype=np.uint8)
        self.L.wfr_set_not_write(self.h, _p(f, C.c_uint8))

    def set_contact(self, mu_static, mu_dynamic):
        self.L.wfr_set_contact(self.h, float(mu_static), float(mu_dynamic))

    def add_trimesh(self, nodes, tris, zone_id, first, vel, angvel=(0.0, 0.0, 0.0), normals=None):
        nd = np.ascontiguousarray(nodes, dtype=np.float64).reshape(-1, 3)
        tr = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
        na = None if normals is None else np.ascontiguousarray(normals, dtype=np.float64)
        v = np.ascontiguousarray(vel, dtype=np.float64)
        w = np.ascontiguousarray(angvel, dtype=np.float64)
        self.L.wfr_add_trimesh(self.h, _p(nd), len(nd), _p(tr, C.c_int32), len(tr),
                               None if na is None else _p(na), int(zone_id), int(first), _p(v),
                               _p(w))

    def get_id(self):
        out = np.empty(self.n, dtype=np.int32)
        self.L.wfr_get_id(self.h, _p(out, C.c_int32))
        return out

    def begin(self):
        self.L.wfr_begin(self.h)

    def thermal_solve(self, sc, nsteps):
        """Domain_d::ThermalSolve's loop (Thermal.cu:188-260) for nsteps steps on a
        heat scenario (positions, masses, density, h, k, c_p, T, BC_T, h_conv, T_inf)."""
        n = self.n
        from weldformgpu_gb300 import _abi as A
        mat = A.WfMaterial(model=A.WF_BILINEAR, E=1.0, nu=0.3)
        self.setup(sc["x"], sc["m"], np.zeros(n, np.int32), sc["h"], sc["rho"], 1.0, 1.0, 1.0,
                   sc["dt"], 1.0, 0.0, mat, T=sc["T"])
        k = np.full(n, float(sc["k"]))
        cp = np.full(n, float(sc["cp"]))
        bc = np.ascontiguousarray(sc["bc_t"], dtype=np.int32)
        self.L.wfr_thermal_solve(self.h, int(nsteps), _p(k), _p(cp), _p(bc, C.c_int32),
                                 float(sc["h_conv"]), float(sc["T_inf"]))

    def step(self, k):
        self.L.wfr_step(self.h, int(k))

    def get(self, name):
        c = _abi.FIELD_COMPONENTS.get(name, 1)
        out = np.empty(self.n * c, dtype=np.float64)
        rc = self.L.wfr_get(self.h, name.encode(), _p(out))
        assert rc == 0, name
        return out.reshape(self.n, c) if c > 1 else out
