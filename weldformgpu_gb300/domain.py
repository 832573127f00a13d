"""Python host binding of libweldform_gb300.so.

`Domain_d` mirrors the reference's SPH::Domain_d (src/cuda/Domain_d.cuh:101-426):
the same setters (Set_h, SetDensity, SetShearModulus, SetSigmay, SetCs,
SetFreePart, SetID, SetConductivity, SetHeatCap) and solve entry points
(MechFraserSolve, MechSolve, ThermalSolve, WriteCSV), plus snake_case names
matching the C ABI one to one.  There is no CPU fallback: if the CUDA
library is missing or no GPU is visible, construction raises.
"""
import ctypes as C
import os

import numpy as np

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libweldform_gb300.so")

_lib = None


class WeldformError(RuntimeError):
    """A C ABI call returned a negative status."""

    def __init__(self, code, what, detail):
        self.code = code
        super().__init__("%s failed: %s (%s)" % (what, _abi.ERROR_NAMES.get(code, code), detail))


def lib():
    """Loads the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("weldformgpu_gb300: CUDA library %s is missing; build it with "
                               "`python -m weldformgpu_gb300.build`" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        _abi.bind(L, "wf_", _abi.SIGNATURES)
        _abi.bind(L, "wf_", _abi.PRODUCT_ONLY)
        _lib = L
    return _lib


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Domain_d:
    """One simulation domain on the GPU (SetDimension == construction)."""

    def __init__(self, particle_count):
        self.L = lib()
        self.h = C.c_void_p()
        rc = self.L.wf_create(C.byref(self.h), int(particle_count))
        if rc != 0:
            raise WeldformError(rc, "wf_create", "no usable CUDA device or allocation failed")
        self.n = int(particle_count)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.wf_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc != 0:
            raise WeldformError(rc, what, self.L.wf_last_error(self.h).decode())

    # ---- scalar setters -------------------------------------------------
    def set_h(self, h): self._ck(self.L.wf_set_h(self.h, float(h)), "wf_set_h")
    def set_density(self, rho): self._ck(self.L.wf_set_density(self.h, float(rho)), "wf_set_density")
    def set_shear_modulus(self, G): self._ck(self.L.wf_set_shear_modulus(self.h, float(G)), "wf_set_shear_modulus")
    def set_sigma_y(self, sy): self._ck(self.L.wf_set_sigma_y(self.h, float(sy)), "wf_set_sigma_y")
    def set_conductivity(self, k): self._ck(self.L.wf_set_conductivity(self.h, float(k)), "wf_set_conductivity")
    def set_heat_cap(self, cp): self._ck(self.L.wf_set_heat_cap(self.h, float(cp)), "wf_set_heat_cap")
    def set_time_step(self, dt): self._ck(self.L.wf_set_time_step(self.h, float(dt)), "wf_set_time_step")
    def set_solid_count(self, n): self._ck(self.L.wf_set_solid_count(self.h, int(n)), "wf_set_solid_count")

    def set_artificial_viscosity(self, alpha, beta):
        self._ck(self.L.wf_set_artificial_viscosity(self.h, float(alpha), float(beta)),
                 "wf_set_artificial_viscosity")

    def set_material(self, mat):
        self._ck(self.L.wf_set_material(self.h, C.byref(mat)), "wf_set_material")

    def add_velocity_bc(self, zone, vx, vy, vz):
        self._ck(self.L.wf_add_velocity_bc(self.h, int(zone), float(vx), float(vy), float(vz)),
                 "wf_add_velocity_bc")

    def set_velocity_bc(self, index, vx, vy, vz):
        """Velocity of BC `index` (wf_add_velocity_bc order), e.g. from the step callback."""
        self._ck(self.L.wf_set_velocity_bc(self.h, int(index), float(vx), float(vy), float(vz)),
                 "wf_set_velocity_bc")

    def set_callback(self, fn):
        """Per-step host hook (the reference's GeneralAfter): fn(domain) after every step;
        a non-zero return ends the solve.  None removes it."""
        if fn is None:
            self._cb = None
            self._ck(self.L.wf_set_callback(self.h, None, None), "wf_set_callback")
            return

        def tramp(_h, _u):
            try:
                r = fn(self)
                return int(r or 0)
            except Exception:          # an exception in the hook ends the solve
                return 1
        self._cb = _abi.AFTER_FN(tramp)
        self._ck(self.L.wf_set_callback(self.h, C.cast(self._cb, C.c_void_p), None),
                 "wf_set_callback")

    def set_contact(self, mu_static, mu_dynamic, law=0):
        self._ck(self.L.wf_set_contact(self.h, float(mu_static), float(mu_dynamic), int(law)),
                 "wf_set_contact")

    def add_trimesh(self, nodes, tris, zone_id, first, vel, angvel=(0.0, 0.0, 0.0), normals=None):
        """Rigid triangle mesh; its element centroids become particles first.. (mass 0)."""
        nd = np.ascontiguousarray(nodes, dtype=np.float64).reshape(-1, 3)
        tr = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
        na = None if normals is None else np.ascontiguousarray(normals, dtype=np.float64)
        nr = None if na is None else _ptr(na, C.c_double)
        v = np.ascontiguousarray(vel, dtype=np.float64)
        w = np.ascontiguousarray(angvel, dtype=np.float64)
        self._ck(self.L.wf_add_trimesh(self.h, _ptr(nd, C.c_double), len(nd), _ptr(tr, C.c_int32),
                                       len(tr), nr, int(zone_id), int(first), _ptr(v, C.c_double),
                                       _ptr(w, C.c_double)), "wf_add_trimesh")

    def set_convection(self, h_conv, T_inf):
        self._ck(self.L.wf_set_convection(self.h, float(h_conv), float(T_inf)), "wf_set_convection")

    def set_option(self, key, value):
        self._ck(self.L.wf_set_option(self.h, key.encode(), float(value)), "wf_set_option(%s)" % key)

    # ---- per-particle setters (caller's particle order) ----------------
    def _d(self, name, a, comps):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        if a.size != comps * self.n:
            raise ValueError("%s: expected %d values, got %d" % (name, comps * self.n, a.size))
        self._ck(getattr(self.L, "wf_" + name)(self.h, _ptr(a, C.c_double)), "wf_" + name)

    def set_positions(self, x): self._d("set_positions", x, 3)
    def set_velocities(self, v): self._d("set_velocities", v, 3)
    def set_mass(self, m): self._d("set_mass", m, 1)
    def set_cs(self, cs): self._d("set_cs", cs, 1)
    def set_temperature(self, T): self._d("set_temperature", T, 1)

    def set_id(self, ids):
        a = np.ascontiguousarray(ids, dtype=np.int32)
        self._ck(self.L.wf_set_id(self.h, _ptr(a, C.c_int32)), "wf_set_id")

    def set_thermal_bc(self, bc):
        a = np.ascontiguousarray(bc, dtype=np.int32)
        self._ck(self.L.wf_set_thermal_bc(self.h, _ptr(a, C.c_int32)), "wf_set_thermal_bc")

    def set_free(self, f):
        a = np.ascontiguousarray(f, dtype=np.uint8)
        self._ck(self.L.wf_set_free(self.h, _ptr(a, C.c_uint8)), "wf_set_free")

    def set_not_write_surf_id(self, f):
        a = np.ascontiguousarray(f, dtype=np.uint8)
        self._ck(self.L.wf_set_not_write_surf_id(self.h, _ptr(a, C.c_uint8)),
                 "wf_set_not_write_surf_id")

    # ---- solvers --------------------------------------------------------
    def mech_fraser_solve(self, tf, dt_out):
        self._ck(self.L.wf_mech_fraser_solve(self.h, float(tf), float(dt_out)), "wf_mech_fraser_solve")

    def mech_solve(self, tf, dt_out):
        self._ck(self.L.wf_mech_solve(self.h, float(tf), float(dt_out)), "wf_mech_solve")

    def thermal_solve(self, tf):
        self._ck(self.L.wf_thermal_solve(self.h, float(tf)), "wf_thermal_solve")

    def step(self, nsteps):
        self._ck(self.L.wf_step(self.h, int(nsteps)), "wf_step")

    def find_neighbors(self):
        self._ck(self.L.wf_find_neighbors(self.h), "wf_find_neighbors")

    def time_steps(self, nsteps):
        """Returns (elapsed_ms, profiled_kernel_ms, profiled_launches, total_launches)."""
        e, k = C.c_double(), C.c_double()
        kl, tl = C.c_int64(), C.c_int64()
        self._ck(self.L.wf_time_steps(self.h, int(nsteps), C.byref(e), C.byref(k), C.byref(kl),
                                      C.byref(tl)), "wf_time_steps")
        return e.value, k.value, kl.value, tl.value

    # ---- outputs --------------------------------------------------------
    def get_field(self, name, out=None):
        """A state field in the caller's order; `out` (float64, n x components,
        C-contiguous, e.g. in pinned host memory) receives it if given."""
        c = _abi.FIELD_COMPONENTS.get(name, 1)
        if out is None:
            out = np.empty(self.n * c, dtype=np.float64)
        elif out.dtype != np.float64 or out.size != self.n * c or not out.flags.c_contiguous:
            raise ValueError("get_field(%s): out must be %d contiguous float64" % (name, self.n * c))
        self._ck(self.L.wf_get_field(self.h, name.encode(), _ptr(out, C.c_double)),
                 "wf_get_field(%s)" % name)
        return out.reshape(self.n, c) if c > 1 else out.reshape(self.n)

    def set_field(self, name, values):
        """Writes a state field (caller's order); see wf_set_field."""
        c = _abi.FIELD_COMPONENTS.get(name, 1)
        self._d_named("set_field", name, values, c)

    def _d_named(self, fn, name, a, comps):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        if a.size != comps * self.n:
            raise ValueError("%s: expected %d values, got %d" % (name, comps * self.n, a.size))
        self._ck(getattr(self.L, "wf_" + fn)(self.h, name.encode(), _ptr(a, C.c_double)),
                 "wf_%s(%s)" % (fn, name))

    def set_mlp_weights(self, params):
        """Loads warm-start MLP parameters (enable with set_option("mlp", 1))."""
        from . import mlp
        mlp.set_domain_weights(self, params)

    def get_return_map_log(self, cap):
        """(features, targets) logged by the plain form under option log_return_map."""
        from . import mlp
        return mlp.get_return_map_log(self, cap)

    def set_scalar(self, name, value):
        self._ck(self.L.wf_set_scalar(self.h, name.encode(), float(value)), "wf_set_scalar(%s)" % name)

    CHECKPOINT_FIELDS = ("x", "m", "v", "rho", "u", "a", "sigma", "shearstress", "strain",
                         "pl_strain", "sigma_y", "int_energy", "T", "Ta", "Tb", "dep")

    def checkpoint(self):
        """All state needed to continue a run, as host arrays."""
        st = {f: self.get_field(f) for f in self.CHECKPOINT_FIELDS}
        st["ID"] = self.get_field_i32("ID")
        for s in ("time", "step", "isfirst", "is_yielding"):
            st["_" + s] = self.get_scalar(s)
        return st

    def restore(self, st):
        """Loads a checkpoint() into this domain; the next solve resumes from it."""
        for f in self.CHECKPOINT_FIELDS:
            self.set_field(f, st[f])
        self.set_id(st["ID"])
        for s in ("time", "step", "isfirst", "is_yielding"):
            self.set_scalar(s, st["_" + s])
        self.set_option("resume", 1)

    def get_field_i32(self, name):
        out = np.empty(self.n, dtype=np.int32)
        self._ck(self.L.wf_get_field_i32(self.h, name.encode(), _ptr(out, C.c_int32)),
                 "wf_get_field_i32(%s)" % name)
        return out

    def get_neighbors(self):
        cnt = np.empty(self.n, dtype=np.int32)
        lst = np.empty(self.n * _abi.WF_MAX_NEIGHBORS, dtype=np.int32)
        self._ck(self.L.wf_get_neighbors(self.h, _ptr(cnt, C.c_int32), _ptr(lst, C.c_int32)),
                 "wf_get_neighbors")
        return cnt, lst.reshape(self.n, _abi.WF_MAX_NEIGHBORS)

    def get_output_series(self):
        """The output rows recorded by the solve (n_rows x width, FP64): time, step,
        max u (3), max pl_strain, contact force sum, contact force vector (3),
        internal energy, then per velocity BC the reaction of its zone (3)."""
        n, w = C.c_int64(), C.c_int64()
        self._ck(self.L.wf_get_output_series(self.h, None, 0, C.byref(n), C.byref(w)),
                 "wf_get_output_series")
        rows = np.empty((n.value, w.value), dtype=np.float64)
        if n.value:
            self._ck(self.L.wf_get_output_series(self.h, _ptr(rows, C.c_double), n.value,
                                                 C.byref(n), C.byref(w)), "wf_get_output_series")
        return rows

    def get_output_row(self):
        w = C.c_int64()
        self._ck(self.L.wf_get_output_row(self.h, None, 0, C.byref(w)), "wf_get_output_row")
        row = np.empty(w.value, dtype=np.float64)
        self._ck(self.L.wf_get_output_row(self.h, _ptr(row, C.c_double), w.value, C.byref(w)),
                 "wf_get_output_row")
        return row

    def get_reaction(self, bc_index=0):
        f = np.empty(3, dtype=np.float64)
        self._ck(self.L.wf_get_reaction(self.h, int(bc_index), _ptr(f, C.c_double)),
                 "wf_get_reaction")
        return f

    def get_scalar(self, name):
        out = C.c_double()
        self._ck(self.L.wf_get_scalar(self.h, name.encode(), C.byref(out)), "wf_get_scalar(%s)" % name)
        return out.value

    def set_csv_output(self, prefix):
        """MechFraserSolve's snapshots: <prefix>out_<time>.csv at the solve start and at
        every output time, and the output rows to <prefix>outputs.csv at its end;
        None turns them off."""
        p = None if prefix is None else str(prefix).encode()
        self._ck(self.L.wf_set_csv_output(self.h, p), "wf_set_csv_output")

    def write_csv(self, path):
        self._ck(self.L.wf_write_csv(self.h, str(path).encode()), "wf_write_csv")

    # ---- the reference's member names (src/cuda/Domain_d.cuh:305-398) ---
    Set_h = set_h
    SetDensity = set_density
    SetShearModulus = set_shear_modulus
    SetSigmay = set_sigma_y
    SetConductivity = set_conductivity
    SetHeatCap = set_heat_cap
    SetCs = set_cs
    SetFreePart = set_free
    SetID = set_id
    MechFraserSolve = mech_fraser_solve
    MechSolve = mech_solve
    ThermalSolve = thermal_solve
    WriteCSV = write_csv


def release_cache():
    """wf_release_cache: frees the device arena that wf_destroy keeps for the
    next domain (e.g. before handing the GPU's memory to another library)."""
    rc = lib().wf_release_cache()
    if rc != 0:
        raise WeldformError(rc, "wf_release_cache", "")


def version():
    return lib().wf_version().decode()
