"""Scenario helpers for the tests: the package's scenario builders plus the
loader for the reference compiled for the CPU (oracle/_ref)."""
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
