"""Generates the golden vectors under tests/golden/ from the reference itself.

The reference's own kernel sources (cuNSearch's neighbour kernels and
Domain_d's CalcDensInc / CalcRateTensors / StressStrainOne / CalcAccel /
UpdatePosFraser / ..., Thermal.cu's heat kernels) are compiled for the CPU by oracle/build_ref.py and
run sequentially in MechFraserSolve's order (oracle/ref_domain.cpp).  This
script drives them on small seeded scenarios and stores the outputs, so that
the oracle (and through it the GPU path) can be checked on machines without
the reference tree.

Usage: python tests/golden/make_golden.py        (needs the reference tree)
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, oracle as O  # noqa: E402
from tests import scenarios as S  # noqa: E402

FIELDS = ["x", "v", "a", "rho", "drho", "p", "sigma", "shearstress", "strrate", "rotrate",
          "sigma_eq", "pl_strain", "sigma_y", "eff_strain_rate", "int_energy"]


def list_digest(cnt, lst):
    """per-particle (sum, sum of squares) of neighbour ids and one sha256 of all lists"""
    n = len(cnt)
    s1 = np.zeros(n, np.int64)
    s2 = np.zeros(n, np.int64)
    h = hashlib.sha256()
    for i in range(n):
        row = lst[i, :cnt[i]].astype(np.int64)
        s1[i] = row.sum()
        s2[i] = (row * row).sum()
        h.update(row.astype(np.int32).tobytes())
    return s1, s2, h.hexdigest()


def run_fraser(sc, checkpoints):
    R = S.load_ref(O.RefDomain(sc["n"]), sc)
    R.begin()
    out = {}
    done = 0
    for k in checkpoints:
        R.step(k - done)
        done = k
        for f in FIELDS + (CONTACT_FIELDS if "mesh" in sc else []):
            out["s%d_%s" % (k, f)] = R.get(f)
        if "mesh" in sc:
            out["s%d_ID" % k] = R.get_id()
    return out


CONTACT_FIELDS = ["u", "normal", "contforce"]


def run_thermal(checkpoints):
    """ThermalSolve on the 16^3 heat box, one fresh run per checkpoint (steps)."""
    hb = S.heat_box(n_side=16)
    out = {}
    for k in checkpoints:
        R = O.RefDomain(hb["n"])
        R.thermal_solve(hb, k)
        for f in ("T", "Ta", "Tb", "dTdt"):
            out["s%d_%s" % (k, f)] = R.get(f)
    return out


def main():
    lib = build_ref.build()
    if lib is None:
        print("reference tree not found; golden vectors not regenerated")
        return 1
    # 1. neighbour lists, small cylinder (reference generator, 540 particles)
    sc = S.compression_cylinder()
    cnt, lst = O.ref_neighbors(sc["x"], sc["h"])
    np.savez_compressed(os.path.join(HERE, "nb_small.npz"), x=sc["x"], h=sc["h"], counts=cnt,
                        lists=lst)
    # 2. neighbour digest of the R = 5 mm, H = 10 mm cylinder (5,244 particles)
    c1 = S.compression_cylinder(R=0.005, H=0.010)
    cnt1, lst1 = O.ref_neighbors(c1["x"], c1["h"])
    s1, s2, dig = list_digest(cnt1, lst1)
    np.savez_compressed(os.path.join(HERE, "nb_c1.npz"), counts=cnt1, sum=s1, sumsq=s2,
                        sha256=np.array(dig), n=c1["n"])
    # 3. Fraser loop, bilinear compression (v_top = -1 m/s): elastic, first
    #    yield and the neighbour rebuilds that follow it
    np.savez_compressed(os.path.join(HERE, "fraser_bilinear.npz"),
                        **run_fraser(sc, [1, 600, 1500]))
    # 4. Fraser loop, Johnson-Cook material (reference radial return), v_top = -10 m/s
    jc = S.compression_cylinder(material="jc", vz_top=-10.0)
    np.savez_compressed(os.path.join(HERE, "fraser_jc.npz"), **run_fraser(jc, [300]))
    # 5. Hollomon power law (reference radial return), v_top = -10 m/s
    ho = S.compression_cylinder(material="hollomon", vz_top=-10.0)
    np.savez_compressed(os.path.join(HERE, "fraser_hollomon.npz"), **run_fraser(ho, [300]))
    # 6. contact: the small cylinder compressed by a rigid plane at -10 m/s
    #    (surface tagging, contact lists, penalty law with friction, mesh motion)
    ct = S.contact_cylinder(R=0.0025, H=0.005, dens=6, mu=(0.3, 0.2))
    np.savez_compressed(os.path.join(HERE, "fraser_contact.npz"),
                        **run_fraser(ct, [1, 200, 600]))
    # 7. heat conduction only (ThermalSolve): 16^3 steel box, Gaussian hot
    #    spot, convection on the outer layer; the reference's ThermalSolveKernel,
    #    CalcConvHeatKernel and TempCalcLeapfrog[First] (src/cuda/Thermal.cu:16-142)
    np.savez_compressed(os.path.join(HERE, "thermal_box.npz"), **run_thermal([1, 100, 500]))
    print("golden vectors written to", HERE)
    return 0


if __name__ == "__main__":
    sys.exit(main())
