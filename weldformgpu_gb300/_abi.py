"""ctypes description of the C ABI in include/weldform_gb300.h.

Shared by the product binding (weldformgpu_gb300.domain) and by the test
oracle's binding, which exports the same entry points with a `wfo_` prefix.
"""
import ctypes as C

WF_OK = 0
WF_ERR_ARG = -1
WF_ERR_CUDA = -2
WF_ERR_STATE = -3
WF_ERR_ALLOC = -4
WF_ERR_NUMERIC = -5
WF_ERR_IO = -6
WF_MAX_NEIGHBORS = 70

WF_BILINEAR = 0
WF_HOLLOMON = 1
WF_JOHNSON_COOK = 2

ERROR_NAMES = {
    WF_ERR_ARG: "WF_ERR_ARG",
    WF_ERR_CUDA: "WF_ERR_CUDA",
    WF_ERR_STATE: "WF_ERR_STATE",
    WF_ERR_ALLOC: "WF_ERR_ALLOC",
    WF_ERR_NUMERIC: "WF_ERR_NUMERIC",
    WF_ERR_IO: "WF_ERR_IO",
}


class WfMaterial(C.Structure):
    """struct wf_material (material constants in the reference's JSON order)."""

    _fields_ = [
        ("model", C.c_int32),
        ("reserved", C.c_int32),
        ("E", C.c_double),
        ("nu", C.c_double),
        ("sy0", C.c_double),
        ("Et", C.c_double),
        ("K_hol", C.c_double),
        ("m_hol", C.c_double),
        ("A", C.c_double),
        ("B", C.c_double),
        ("n", C.c_double),
        ("C", C.c_double),
        ("eps0", C.c_double),
        ("m", C.c_double),
        ("Tm", C.c_double),
        ("Tt", C.c_double),
    ]


_d = C.c_double
_i64 = C.c_int64
_i32 = C.c_int32
_vp = C.c_void_p
_pd = C.POINTER(C.c_double)
_pi32 = C.POINTER(C.c_int32)
_pu8 = C.POINTER(C.c_uint8)
_cs = C.c_char_p

# name -> (restype, argtypes); names without the wf_/wfo_ prefix.
SIGNATURES = {
    "create": (C.c_int, [C.POINTER(_vp), _i64]),
    "destroy": (C.c_int, [_vp]),
    "last_error": (C.c_char_p, [_vp]),
    "set_h": (C.c_int, [_vp, _d]),
    "set_density": (C.c_int, [_vp, _d]),
    "set_shear_modulus": (C.c_int, [_vp, _d]),
    "set_sigma_y": (C.c_int, [_vp, _d]),
    "set_conductivity": (C.c_int, [_vp, _d]),
    "set_heat_cap": (C.c_int, [_vp, _d]),
    "set_cs": (C.c_int, [_vp, _pd]),
    "set_free": (C.c_int, [_vp, _pu8]),
    "set_id": (C.c_int, [_vp, _pi32]),
    "set_positions": (C.c_int, [_vp, _pd]),
    "set_velocities": (C.c_int, [_vp, _pd]),
    "set_mass": (C.c_int, [_vp, _pd]),
    "set_not_write_surf_id": (C.c_int, [_vp, _pu8]),
    "set_solid_count": (C.c_int, [_vp, _i64]),
    "set_time_step": (C.c_int, [_vp, _d]),
    "set_artificial_viscosity": (C.c_int, [_vp, _d, _d]),
    "set_material": (C.c_int, [_vp, C.POINTER(WfMaterial)]),
    "add_velocity_bc": (C.c_int, [_vp, _i32, _d, _d, _d]),
    "set_velocity_bc": (C.c_int, [_vp, _i32, _d, _d, _d]),
    "get_output_series": (C.c_int, [_vp, _pd, _i64, C.POINTER(_i64), C.POINTER(_i64)]),
    "set_temperature": (C.c_int, [_vp, _pd]),
    "set_thermal_bc": (C.c_int, [_vp, _pi32]),
    "set_convection": (C.c_int, [_vp, _d, _d]),
    "set_option": (C.c_int, [_vp, _cs, _d]),
    "mech_fraser_solve": (C.c_int, [_vp, _d, _d]),
    "thermal_solve": (C.c_int, [_vp, _d]),
    "step": (C.c_int, [_vp, _i64]),
    "find_neighbors": (C.c_int, [_vp]),
    "get_field": (C.c_int, [_vp, _cs, _pd]),
    "get_field_i32": (C.c_int, [_vp, _cs, _pi32]),
    "get_neighbors": (C.c_int, [_vp, _pi32, _pi32]),
    "get_scalar": (C.c_int, [_vp, _cs, _pd]),
    "set_field": (C.c_int, [_vp, _cs, _pd]),
    # contact with rigid triangle meshes
    "set_contact": (C.c_int, [_vp, _d, _d, C.c_int]),
    "add_trimesh": (C.c_int, [_vp, _pd, _i32, _pi32, _i32, _pd, _i32, _i64, _pd, _pd]),
    "gen_plane_mesh": (_i64, [C.c_int, C.c_int, _pd, _pd, C.c_int, _pd, _pi32, _pd]),
}

# entry points without a domain handle
NO_HANDLE = {"gen_plane_mesh"}

# entry points only the product exports
PRODUCT_ONLY = {
    "version": (C.c_char_p, []),
    "mech_solve": (C.c_int, [_vp, _d, _d]),
    "write_csv": (C.c_int, [_vp, _cs]),
    "set_csv_output": (C.c_int, [_vp, _cs]),
    "set_scalar": (C.c_int, [_vp, _cs, _d]),
    "time_steps": (C.c_int, [_vp, _i64, _pd, _pd, C.POINTER(_i64), C.POINTER(_i64)]),
    "get_output_row": (C.c_int, [_vp, _pd, _i64, C.POINTER(_i64)]),
    "get_reaction": (C.c_int, [_vp, _i32, _pd]),
    "set_callback": (C.c_int, [_vp, _vp, _vp]),
    "fp64_fma_peak": (C.c_int, [_pd, _pd]),
}

# int (*wf_after_fn)(wf_domain*, void*): the per-step host hook
AFTER_FN = C.CFUNCTYPE(C.c_int, _vp, _vp)

# columns of an output row before the per-BC reactions (WF_ROW_FIXED_COLUMNS)
ROW_FIXED = 11
ROW_COLUMNS = ("time", "step", "max_ux", "max_uy", "max_uz", "max_pl_strain", "cont_force_sum",
               "cont_fx", "cont_fy", "cont_fz", "int_energy")

FIELD_COMPONENTS = {
    "x": 3, "v": 3, "a": 3, "u": 3, "normal": 3, "contforce": 3,
    "sigma": 6, "strrate": 6, "rotrate": 6, "shearstress": 6, "strain": 6,
}


def bind(lib, prefix, names):
    """Attach restype/argtypes to `lib.<prefix><name>` for every name."""
    for name, (res, args) in names.items():
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
    return lib
