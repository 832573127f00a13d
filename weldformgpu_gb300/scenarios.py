"""Synthetic scenarios with the shapes of the benchmark configurations.

A scenario is a plain dict (positions, masses, ids, scalars, material, BCs)
that `load()` applies through the Domain_d setters.  The generators are the
reference's (src/Domain.cpp) as implemented by the library, plus the seeded
jittered lattice the benchmark configurations use.
"""
import math

import numpy as np

from . import _abi
from . import setup as S
from . import setup as _gen


def compression_cylinder(R=0.0025, H=0.005, dx=0.0005, generator="reference", vz_top=-1.0,
                         material="bilinear", jitter=0.01, seed=1, layers=2, dt_rule="reference",
                         gen=None):
    """Elastoplastic cylinder compression (the reference's Compression example
    shape; the 5,000-step benchmark case is R=5 mm, H=10 mm).  Bottom `layers` layers are
    fixed (zone 2), top `layers` layers move at vz_top (zone 3).  `gen` supplies
    gen_cylinder_ref / gen_cylinder_lattice / assign_zone (default: the
    library's; any module with the same functions, e.g. a CPU twin)."""
    S = gen if gen is not None else _gen
    r = dx / 2.0
    rho = 2700.0
    if generator == "reference":
        x, mass = S.gen_cylinder_ref((0.0, 0.0, 0.0), R, H, r, rho)
        m = np.full(len(x), mass)
    else:
        x = S.gen_cylinder_lattice(R, H, dx, jitter, seed)
        m = np.full(len(x), rho * dx ** 3)
    n = len(x)
    if material == "bilinear":
        E, nu = 70e9, 0.33
        mat = _abi.WfMaterial(model=_abi.WF_BILINEAR, E=E, nu=nu, sy0=300e6, Et=700e6)
        sy = 300e6
        T0 = 20.0
    elif material == "hollomon":   # power law K (eps + eps0)^m with a plateau at sy0
        E, nu = 70e9, 0.33
        mat = _abi.WfMaterial(model=_abi.WF_HOLLOMON, E=E, nu=nu, sy0=300e6, K_hol=500e6,
                              m_hol=0.2)
        sy = 300e6
        T0 = 20.0
    else:  # Johnson-Cook aluminium: A 324 MPa, B 114 MPa, n 0.42, C 0.002, m 1.34, Tm 582 C
        E, nu = 70e9, 0.33
        mat = _abi.WfMaterial(model=_abi.WF_JOHNSON_COOK, E=E, nu=nu, sy0=324e6, A=324e6,
                              B=114e6, n=0.42, C=0.002, eps0=1.0, m=1.34, Tm=582.0, Tt=20.0)
        sy = 324e6
        T0 = 20.0
    K = E / (3.0 * (1.0 - 2.0 * nu))
    G = E / (2.0 * (1.0 + nu))
    Cs = math.sqrt(K / rho)
    h = 1.2 * dx
    if dt_rule == "reference":       # src/WeldFormGPU.cu:906, VMAX = 10
        dt = 0.4 * h / (Cs + 10.0)
    else:                            # 0.4 h / c (c = sqrt(K / rho))
        dt = 0.4 * h / Cs
    ids = np.zeros(n, np.int32)
    nw = np.zeros(n, np.uint8)
    zmin, zmax = x[:, 2].min(), x[:, 2].max()
    S.assign_zone(x, (-1, -1, -1), (1, 1, zmin + (layers - 0.5) * dx), 2, ids, nw)
    S.assign_zone(x, (-1, -1, zmax - (layers - 0.5) * dx), (1, 1, 1), 3, ids, nw)
    return dict(n=n, x=x, m=m, ids=ids, not_write=nw, h=h, rho=rho, G=G, sy=sy, Cs=Cs, dt=dt,
                alpha=1.0, beta=0.0, mat=mat, T=np.full(n, T0),
                bcs=[(2, (0.0, 0.0, 0.0)), (3, (0.0, 0.0, vz_top))], K=K, dx=dx)


def contact_cylinder(R=0.005, H=0.010, dx=0.0005, dens=10, v_plane=-10.0, gap=1.0e-7,
                     mu=(0.0, 0.0), material="bilinear", zone=5):
    """Cylinder (the reference generator) with its bottom two layers fixed,
    compressed by a rigid plane from above, as main sets up a "Plane" rigid
    body (src/WeldFormGPU.cu:498-610): AxisPlaneMesh(2, false, ...) with
    `dens` cells a side, normal -z, starting `gap` beyond contact range (one
    smoothing length above the top particles) and moving at v_plane; its
    2 dens^2 element centroids are the last particles (zone `zone`)."""
    sc = compression_cylinder(R=R, H=H, dx=dx, material=material)
    x_s = sc["x"]
    ns = len(x_s)
    ids = np.zeros(ns, np.int32)
    nw = np.zeros(ns, np.uint8)
    zmin, zmax = x_s[:, 2].min(), x_s[:, 2].max()
    S.assign_zone(x_s, (-1, -1, -1), (1, 1, zmin + 1.5 * dx), 2, ids, nw)
    side = 2.0 * R + 2.0 * dx
    p1 = (-R - dx, -R - dx, zmax + sc["h"] + gap)
    p2 = (p1[0] + side, p1[1] + side, p1[2])
    nodes, tris, normals = S.gen_plane_mesh(2, 0, p1, p2, dens)
    ne = len(tris)
    n = ns + ne
    sc.update(
        n=n, n_solid=ns,
        x=np.vstack([x_s, np.zeros((ne, 3))]),
        m=np.concatenate([sc["m"], np.zeros(ne)]),
        ids=np.concatenate([ids, np.full(ne, zone, np.int32)]),
        not_write=np.concatenate([nw, np.zeros(ne, np.uint8)]),
        T=np.full(n, 20.0),
        bcs=[(2, (0.0, 0.0, 0.0)), (zone, (0.0, 0.0, v_plane))],
        mesh=dict(nodes=nodes, tris=tris, normals=normals, zone=zone, first=ns,
                  vel=(0.0, 0.0, v_plane), angvel=(0.0, 0.0, 0.0)),
        mu=mu)
    return sc


def indent_block(L=(0.008, 0.008, 0.003), dx=0.00025, R=0.003, level=3, v_tool=-5.0, mu=0.3,
                 gap=1.0e-7, thermal=True, zone=7, rebuild_increment=0.05, omega=0.0):
    """A block indented by a rigid lower-half icosphere (the shape of the
    2M-particle contact benchmark: block 200 x 200 x 50 dx,
    dx = 0.25 mm, R = 10 mm, ~10k triangles, -5 m/s): contact law 1 (penalty
    0.1 K / dx, friction mu, cell-binned triangle query, frictional heat), JC
    aluminium, neighbour rebuild at a plastic-strain increment.  The bottom
    layer is fixed (zone 2); the tool starts `gap` outside contact range.
    omega != 0 spins the tool about the z axis (rad/s): the block is then
    centred on that axis (x, y in [-L/2, L/2]), as for a stirring tool."""
    rho, E, nu = 2700.0, 70e9, 0.33
    x0 = (-L[0] / 2.0, -L[1] / 2.0, 0.0) if omega != 0.0 else (0.0, 0.0, 0.0)
    x, mass = S.gen_box_cubic(x0, L, dx / 2.0, rho)
    ns = len(x)
    nodes, tris = S.gen_icosphere(R, (0.0, 0.0, 0.0), level, True)
    top = x[:, 2].max()
    cxy = (0.0, 0.0) if omega != 0.0 else (L[0] / 2.0, L[1] / 2.0)
    shift = np.array([cxy[0], cxy[1], top + dx / 2.0 + gap - nodes[:, 2].min()])
    nodes = nodes + shift
    ne = len(tris)
    n = ns + ne
    ids = np.zeros(n, np.int32)
    nw = np.zeros(n, np.uint8)
    S.assign_zone(x, (-1, -1, -1), (1, 1, x[:, 2].min() + 0.5 * dx), 2, ids[:ns], nw[:ns])
    ids[ns:] = zone
    mat = _abi.WfMaterial(model=_abi.WF_JOHNSON_COOK, E=E, nu=nu, sy0=324e6, A=324e6, B=114e6,
                          n=0.42, C=0.002, eps0=1.0, m=1.34, Tm=582.0, Tt=20.0)
    K = E / (3.0 * (1.0 - 2.0 * nu))
    G = E / (2.0 * (1.0 + nu))
    Cs = math.sqrt(K / rho)
    h = 1.2 * dx
    opts = {"contact_dx": dx, "return_map": 1, "rebuild_current_positions": 1,
            "rebuild_strain_increment": rebuild_increment}
    sc = dict(n=n, n_solid=ns, x=np.vstack([x, np.zeros((ne, 3))]),
              m=np.concatenate([np.full(ns, mass), np.zeros(ne)]), ids=ids, not_write=nw,
              h=h, rho=rho, G=G, sy=324e6, Cs=Cs, dt=0.4 * h / Cs, alpha=1.0, beta=0.0, mat=mat,
              T=np.full(n, 20.0), bcs=[(2, (0.0, 0.0, 0.0)), (zone, (0.0, 0.0, v_tool))], K=K,
              dx=dx, mesh=dict(nodes=nodes, tris=tris, normals=None, zone=zone, first=ns,
                               vel=(0.0, 0.0, v_tool), angvel=(0.0, 0.0, omega)),
              mu=(mu, mu), law=1, options=opts)
    if thermal:
        sc["k"], sc["cp"] = 167.0, 896.0
        opts.update(thermal=1, taylor_quinney=0.9)
    return sc


def load(dom, sc, options=None):
    """Applies a scenario through the Domain_d setters (product or oracle)."""
    n = sc["n"]
    if "n_solid" in sc:
        dom.set_solid_count(sc["n_solid"])
    dom.set_h(sc["h"])
    dom.set_density(sc["rho"])
    dom.set_shear_modulus(sc["G"])
    dom.set_sigma_y(sc["sy"])
    cs = sc.get("Cs_particles")          # the per-particle array, when the caller holds one
    dom.set_cs(cs if cs is not None else np.full(n, sc["Cs"]))
    dom.set_positions(np.ascontiguousarray(sc["x"]).ravel())
    dom.set_mass(sc["m"])
    dom.set_id(sc["ids"])
    dom.set_not_write_surf_id(sc["not_write"])
    dom.set_time_step(sc["dt"])
    dom.set_artificial_viscosity(sc["alpha"], sc["beta"])
    dom.set_material(sc["mat"])
    dom.set_temperature(sc["T"])
    for zone, v in sc["bcs"]:
        dom.add_velocity_bc(zone, float(v[0]), float(v[1]), float(v[2]))
    if "k" in sc:
        dom.set_conductivity(sc["k"])
        dom.set_heat_cap(sc["cp"])
    if "mesh" in sc:
        ms = sc["mesh"]
        dom.add_trimesh(ms["nodes"], ms["tris"], ms["zone"], ms["first"], ms["vel"], ms["angvel"],
                        normals=ms["normals"])
        dom.set_contact(sc["mu"][0], sc["mu"][1], sc.get("law", 0))
    for k, v in dict(sc.get("options", {}), **(options or {})).items():
        dom.set_option(k, float(v))
    return dom


def heat_box(n_side=20, dx=1.0e-4, hot=500.0, T0=20.0, sigma=1.0e-3):
    """Heat conduction only (the 100^3-particle heat box's shape at n_side^3 particles):
    steel cube, Gaussian hot spot at the centre, convection on the outer layer."""
    rho, cp, k = 7850.0, 460.0, 50.0
    L = n_side * dx
    x, mass = S.gen_box_cubic((0.0, 0.0, 0.0), (L, L, L), dx / 2.0, rho)
    n = len(x)
    c = 0.5 * L
    r2 = np.sum((x - c) ** 2, axis=1)
    T = T0 + (hot - T0) * np.exp(-r2 / (2.0 * sigma * sigma))
    lo, hi = x.min(axis=0), x.max(axis=0)
    outer = np.any((x <= lo + 0.5 * dx) | (x >= hi - 0.5 * dx), axis=1)
    bc_t = outer.astype(np.int32)
    dt = 0.1 * dx * dx * rho * cp / k
    return dict(n=n, x=x, m=np.full(n, mass), h=1.2 * dx, rho=rho, cp=cp, k=k, T=T, bc_t=bc_t,
                dt=dt, h_conv=100.0, T_inf=T0, dx=dx)


def load_heat(dom, sc):
    n = sc["n"]
    dom.set_h(sc["h"])
    dom.set_density(sc["rho"])
    dom.set_positions(np.ascontiguousarray(sc["x"]).ravel())
    dom.set_mass(sc["m"])
    dom.set_conductivity(sc["k"])
    dom.set_heat_cap(sc["cp"])
    dom.set_temperature(sc["T"])
    dom.set_thermal_bc(sc["bc_t"])
    dom.set_convection(sc["h_conv"], sc["T_inf"])
    dom.set_time_step(sc["dt"])
    return dom


def jc_compression(R=0.025, H=0.050, dx=0.0005, jitter=0.01, seed=1, vz_top=-10.0, layers=2,
                   gen=None):
    """Coupled thermo-mechanical Johnson-Cook compression (R 25 mm, H 50 mm, dx 0.5 mm):
    R = 25 mm, H = 50 mm, dx = 0.5 mm (~0.79M particles), jitter +-0.01 dx,
    JC A=324 MPa, B=114 MPa, n=0.42, C=0.002, m=1.34, eps0=1/s, Tref=20 C,
    Tmelt=582 C; k=167 W/mK, cp=896 J/kgK, Taylor-Quinney 0.9 (set as an
    option by the caller); top `layers` layers at vz_top, bottom ones fixed;
    dt = 0.4 h / c."""
    sc = compression_cylinder(R=R, H=H, dx=dx, generator="lattice", jitter=jitter, seed=seed,
                              vz_top=vz_top, material="jc", layers=layers, dt_rule="sound_speed",
                              gen=gen)
    sc["k"], sc["cp"] = 167.0, 896.0
    return sc
