"""Scenario helpers for the tests: the package's scenario builders plus the
loader for the reference compiled for the CPU (oracle/_ref)."""
import numpy as np

from weldformgpu_gb300.scenarios import *  # noqa: F401,F403
from weldformgpu_gb300.scenarios import compression_cylinder, heat_box, load, load_heat  # noqa: F401


def load_ref(R, sc):
    """Applies a scenario to oracle.oracle.RefDomain (the reference's kernels on the CPU)."""
    R.setup(sc["x"], sc["m"], sc["ids"], sc["h"], sc["rho"], sc["G"], sc["sy"], sc["Cs"],
            sc["dt"], sc["alpha"], sc["beta"], sc["mat"], T=sc["T"])
    for zone, v in sc["bcs"]:
        R.add_bc(zone, v)
    if "mesh" in sc:
        ms = sc["mesh"]
        R.set_not_write(sc["not_write"])
        R.add_trimesh(ms["nodes"], ms["tris"], ms["zone"], ms["first"], ms["vel"], ms["angvel"],
                      normals=ms["normals"])
        R.set_contact(sc["mu"][0], sc["mu"][1])
    return R


def one_particle_under_triangle(x0, tri_nodes, v_tool, mu=0.3, dx=1.0e-3, dt=1.0e-8):
    """Known-answer case for contact law 1: one solid particle at rest (a solve
    starts with the solid velocities zeroed, as the reference's SetVelKernel
    does; no SPH neighbours) and one rigid triangle moving at v_tool.  Returns
    the scenario and the law's closed form for the first step: force, frictional
    heat and contact normal (nearest point on the triangle, penalty
    0.1 K dx delta, friction -mu F_n v_t / max(|v_t|, 1e-3), heat
    mu F_n |v_t|^2 / max(|v_t|, 1e-3))."""
    import math
    import numpy as np
    from weldformgpu_gb300 import _abi
    rho, E, nu = 2700.0, 70e9, 0.33
    m = rho * dx ** 3
    nodes = np.asarray(tri_nodes, dtype=np.float64).reshape(3, 3)
    mat = _abi.WfMaterial(model=_abi.WF_BILINEAR, E=E, nu=nu, sy0=300e6, Et=0.0)
    K = E / (3.0 * (1.0 - 2.0 * nu))
    sc = dict(n=2, n_solid=1, x=np.array([x0, [0.0, 0.0, 0.0]], dtype=np.float64),
              m=np.array([m, 0.0]), ids=np.array([0, 7], np.int32),
              not_write=np.zeros(2, np.uint8), h=1.2 * dx, rho=rho,
              G=E / (2.0 * (1.0 + nu)), sy=300e6, Cs=math.sqrt(K / rho), dt=dt, alpha=1.0,
              beta=0.0, mat=mat, T=np.full(2, 20.0), bcs=[(7, tuple(v_tool))], k=167.0, cp=896.0,
              mesh=dict(nodes=nodes, tris=np.array([[0, 1, 2]], np.int32), normals=None, zone=7,
                        first=1, vel=tuple(v_tool), angvel=(0.0, 0.0, 0.0)),
              mu=(mu, mu), law=1, options={"contact_dx": dx, "thermal": 1})

    def expected(q):
        """Force, frictional heat and normal for the nearest surface point q."""
        x = np.asarray(x0, dtype=np.float64)
        nf = np.cross(nodes[1] - nodes[0], nodes[2] - nodes[0])
        nf /= np.linalg.norm(nf)
        dv = x - np.asarray(q, dtype=np.float64)
        dist = np.linalg.norm(dv)
        if dv @ nf >= 0.0 and dist > 0.0:
            n, g = dv / dist, dist
        else:
            n, g = nf, dv @ nf
        delta = 0.5 * dx - g
        if delta <= 0.0:
            return np.zeros(3), 0.0, n
        fn = 0.1 * K * dx * delta
        vrel = -np.asarray(v_tool, dtype=np.float64)
        vt = vrel - n * (vrel @ n)
        s = mu * fn / max(np.linalg.norm(vt), 1.0e-3)
        return fn * n - s * vt, s * (vt @ vt), n
    return sc, expected


def support_radius_pairs(h=1.0e-3, seed=3):
    """4,000 isolated pairs whose distance lies within +-4e-7 (relative, about
    3 float32 ulps) of the support radius r = 2h."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(np.arange(20), np.arange(20), np.arange(10), indexing="ij"),
                 -1).reshape(-1, 3)
    a = g * (10.0 * h) + rng.uniform(-0.5 * h, 0.5 * h, g.shape)
    u = rng.normal(size=g.shape)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = float(np.float32(2.0 * h))
    e = rng.uniform(-4e-7, 4e-7, len(g))
    x = np.empty((2 * len(g), 3))
    x[0::2] = a
    x[1::2] = a + u * (r * (1.0 + e))[:, None]
    return x
