"""GPU parity: the CUDA path through the C ABI against the oracle and the
reference's golden vectors.

Tolerances:
  - neighbour lists: identical sets and identical order (bit-exact);
  - plain FP64 form, reference radial return: bit-exact (np.array_equal) --
    the FP64 kernels build with -fmad=false and sum neighbours in the
    oracle's order;
  - plain FP64 form with pow/log (Johnson-Cook Newton, convection): 1e-9
    relative, the plain-form bound (CUDA's pow/log may differ
    from glibc's in the last bit);
  - mixed form: relative L2 error <= 1e-3 per output field against the
    plain FP64 run of the same pipeline.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import scenarios as S

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STATE_FIELDS = ["x", "v", "a", "rho", "drho", "p", "sigma", "shearstress", "strrate", "rotrate",
                "sigma_eq", "pl_strain", "sigma_y", "eff_strain_rate", "int_energy"]


def gpu(sc, options=None):
    from weldformgpu_gb300 import Domain_d
    return S.load(Domain_d(sc["n"]), sc, options)


def ora(sc, options=None):
    return S.load(O.OracleDomain(sc["n"]), sc, options)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def same_lists(c1, l1, c2, l2):
    if not np.array_equal(c1, c2):
        return False
    return all(np.array_equal(l1[i, :c1[i]], l2[i, :c2[i]]) for i in range(len(c1)))


def test_neighbors_bit_exact_cylinder_r5mm():
    c1 = S.compression_cylinder(R=0.005, H=0.010)
    g = gpu(c1)
    g.find_neighbors()
    o = ora(c1)
    o.find_neighbors()
    assert same_lists(*g.get_neighbors(), *o.get_neighbors())
    gold = np.load(os.path.join(GOLDEN, "nb_c1.npz"))
    assert np.array_equal(g.get_field_i32("nb_count"), gold["counts"])


def test_neighbors_bit_exact_jittered_lattice():
    sc = S.compression_cylinder(R=0.004, H=0.006, generator="lattice", jitter=0.01, seed=7)
    g = gpu(sc)
    g.find_neighbors()
    o = ora(sc)
    o.find_neighbors()
    assert same_lists(*g.get_neighbors(), *o.get_neighbors())


def test_neighbour_lists_dense_clusters_and_cap():
    """Isolated clusters of 40 particles (cells holding more than a warp's
    worth of particles) and of 90 (lists truncated at 70 entries, the first 70
    in search order, as cuNSearch's CUDA_MAX_NEIGHBORS): lists identical to
    the oracle's, the truncation recorded in bit 2 of the status word."""
    from weldformgpu_gb300 import Domain_d
    h = 1.0e-3
    rng = np.random.default_rng(11)
    pts = []
    for a in range(3):
        for b in range(3):
            for c in range(3):
                size = 90 if (a + b + c) % 4 == 0 else 40
                centre = np.array([a, b, c]) * 3.0 * h    # clusters 2.4 h apart, r = 2 h
                pts.append(centre + rng.uniform(-0.3 * h, 0.3 * h, (size, 3)))
    x = np.vstack(pts)
    n = len(x)
    g = Domain_d(n)
    g.set_h(h)
    g.set_positions(x)
    g.find_neighbors()
    o = O.OracleDomain(n)
    o.set_h(h)
    o.set_positions(np.ascontiguousarray(x).ravel())
    o.find_neighbors()
    gc, gl = g.get_neighbors()
    oc, ol = o.get_neighbors()
    assert same_lists(gc, gl, oc, ol)
    assert gc.max() == 70 and (gc == 39).sum() > 0
    assert int(g.get_scalar("status")) & 2


@pytest.mark.parametrize("case,checkpoints", [("bilinear", [1, 600, 1500]), ("jc", [300]),
                                              ("hollomon", [300])])
def test_fp64_fraser_loop_bit_exact_vs_reference_golden(case, checkpoints):
    gold = np.load(os.path.join(GOLDEN, "fraser_%s.npz" % case))
    sc = (S.compression_cylinder() if case == "bilinear"
          else S.compression_cylinder(material=case, vz_top=-10.0))
    g = gpu(sc)
    done = 0
    for k in checkpoints:
        g.step(k - done)
        done = k
        for f in STATE_FIELDS:
            if case != "bilinear":
                # pow/log of the JC and Hollomon laws: CUDA's and glibc's may differ in
                # the last bit, and that difference reaches every field through the positions
                ref = gold["s%d_%s" % (k, f)]
                np.testing.assert_allclose(g.get_field(f), ref, rtol=1e-9,
                                           atol=1e-9 * np.max(np.abs(ref)))
            else:
                got, ref = g.get_field(f), gold["s%d_%s" % (k, f)]
                assert np.array_equal(got, ref), "%s step %d %s: max |d| %.3e" % (
                    case, k, f, np.max(np.abs(got - ref)))


def test_fp64_cylinder_r5mm_lattice_vs_oracle_with_rebuilds():
    """R 5 mm, H 10 mm jittered lattice, dt 0.4h/c, rebuild every 10 steps, for 400 steps."""
    sc = S.compression_cylinder(R=0.005, H=0.010, generator="lattice", dt_rule="sound_speed")
    opts = {"rebuild_every": 10, "rebuild_current_positions": 1, "rebuild_after_yield": 0}
    g = gpu(sc, opts)
    o = ora(sc, opts)
    g.step(400)
    o.step(400)
    for f in ("x", "u", "v", "rho", "sigma", "pl_strain", "sigma_eq", "int_energy"):
        assert np.array_equal(g.get_field(f), o.get_field(f)), f


def test_fp64_newton_jc_vs_oracle():
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    g = gpu(sc, {"return_map": 1})
    o = ora(sc, {"return_map": 1})
    g.step(400)
    o.step(400)
    assert o.get_field("pl_strain").max() > 0.01
    for f in ("x", "u", "sigma", "pl_strain", "sigma_eq", "sigma_y"):
        ref = o.get_field(f)
        np.testing.assert_allclose(g.get_field(f), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())
    gi = g.get_scalar("newton_iters") / g.get_scalar("newton_calls")
    oi = o.get_scalar("newton_iters") / o.get_scalar("newton_calls")
    assert abs(gi - oi) < 0.05 * oi


def test_mixed_form_within_1e3_of_fp64_jc_newton():
    sc = S.compression_cylinder(R=0.004, H=0.008, material="jc", vz_top=-10.0,
                                generator="lattice", dt_rule="sound_speed")
    opts = {"return_map": 1, "rebuild_every": 10, "rebuild_current_positions": 1,
            "rebuild_after_yield": 0}
    a = gpu(sc, dict(opts, precision=0))
    b = gpu(sc, dict(opts, precision=1))
    a.step(600)
    b.step(600)
    assert a.get_field("pl_strain").max() > 0.005
    for f in ("u", "pl_strain", "sigma_eq"):
        e = rel_l2(b.get_field(f), a.get_field(f))
        assert e <= 1e-3, (f, e)


@pytest.mark.parametrize("mode", [0, 1])
def test_mixed_internal_energy_within_1e3_of_fp64(mode):
    """CalcIntEnergy in both energy modes: 0 (the reference's: particle 0's
    S:D for every particle, Energy.cu:270-276) and 1 (each particle's own),
    the mixed form against plain FP64, and the FP64 form against the oracle."""
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    opts = {"return_map": 1, "energy_mode": mode}
    a = gpu(sc, dict(opts, precision=0))
    b = gpu(sc, dict(opts, precision=1))
    o = ora(sc, opts)
    a.step(300)
    b.step(300)
    o.step(300)
    ea, eb, eo = a.get_field("int_energy"), b.get_field("int_energy"), o.get_field("int_energy")
    assert np.abs(ea).max() > 0
    if mode == 0:      # one S0:D0 per step for every particle, scaled by each m/rho
        assert np.ptp(ea) <= 0.05 * np.abs(ea).max()
    np.testing.assert_allclose(ea, eo, rtol=1e-9, atol=1e-9 * np.abs(eo).max())
    e = rel_l2(eb, ea)
    assert e <= 1e-3, e


def test_heat_fp64_vs_oracle():
    sc = S.heat_box(n_side=16)
    from weldformgpu_gb300 import Domain_d
    g = S.load_heat(Domain_d(sc["n"]), sc)
    o = S.load_heat(O.OracleDomain(sc["n"]), sc)
    tf = 40 * sc["dt"]
    g.thermal_solve(tf)
    o.thermal_solve(tf)
    np.testing.assert_allclose(g.get_field("T"), o.get_field("T"), rtol=1e-12)


@pytest.mark.parametrize("k", [1, 100, 500])
def test_heat_fp64_vs_reference_thermal_golden(k):
    """Heat only on the GPU (plain FP64) against the reference's own
    Thermal.cu kernels (golden vectors, 16^3 box with convection): T, Ta, Tb
    within 1e-12 relative (CUDA's pow in the convection term may differ from
    the host's in the last bit); the rate dT/dt, a sum of differences of
    nearly equal temperatures that amplifies those bits, within the plain
    form's 1e-9."""
    g = np.load(os.path.join(GOLDEN, "thermal_box.npz"))
    sc = S.heat_box(n_side=16)
    from weldformgpu_gb300 import Domain_d
    d = S.load_heat(Domain_d(sc["n"]), sc)
    d.thermal_solve((k - 0.5) * sc["dt"])
    assert d.get_scalar("step") == k
    for f in ("T", "Ta", "Tb"):
        np.testing.assert_allclose(d.get_field(f), g["s%d_%s" % (k, f)], rtol=1e-12, atol=0)
    ref = g["s%d_dTdt" % k]
    np.testing.assert_allclose(d.get_field("dTdt"), ref, rtol=1e-9,
                               atol=1e-9 * np.abs(ref).max())


def test_heat_mixed_flux_vs_fp64():
    sc = S.heat_box(n_side=16)
    from weldformgpu_gb300 import Domain_d
    a = S.load_heat(Domain_d(sc["n"]), sc)
    b = S.load_heat(Domain_d(sc["n"]), sc)
    b.set_option("precision", 1)
    tf = 40 * sc["dt"]
    a.thermal_solve(tf)
    b.thermal_solve(tf)
    T0 = sc["T"]
    assert rel_l2(b.get_field("T") - T0, a.get_field("T") - T0) <= 1e-3


def test_coupled_thermomechanical_jc_vs_oracle():
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    sc["k"], sc["cp"] = 167.0, 896.0
    opts = {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9}
    g = gpu(sc, opts)
    o = ora(sc, opts)
    g.step(300)
    o.step(300)
    To = o.get_field("T")
    assert To.max() > 20.5                         # plastic work heated the cylinder
    np.testing.assert_allclose(g.get_field("T"), To, rtol=1e-9)
    np.testing.assert_allclose(g.get_field("pl_strain"), o.get_field("pl_strain"), rtol=1e-9,
                               atol=1e-12)


def test_contact_fp64_bit_exact_vs_reference_golden():
    """Rigid plane pressing the small cylinder: surface tagging, contact lists,
    penalty law with friction, mesh motion and rigid particles on the GPU,
    against the reference's own contact kernels, bit for bit."""
    g = np.load(os.path.join(GOLDEN, "fraser_contact.npz"))
    sc = S.contact_cylinder(R=0.0025, H=0.005, dens=6, mu=(0.3, 0.2))
    d = gpu(sc)
    done = 0
    for k in (1, 200, 600):
        d.step(k - done)
        done = k
        for f in STATE_FIELDS + ["u", "normal", "contforce"]:
            got, ref = d.get_field(f), g["s%d_%s" % (k, f)]
            assert np.array_equal(got, ref, equal_nan=True), "step %d %s: max |d| %.3e" % (
                k, f, np.nanmax(np.abs(got - ref)))
        assert np.array_equal(d.get_field_i32("ID"), g["s%d_ID" % k])
    assert (np.abs(d.get_field("contforce")).sum(axis=1) > 0).sum() > 20


def test_contact_cylinder_r5mm_fp64_bit_exact_vs_oracle():
    """The R 5 mm, H 10 mm cylinder (5,244 particles) under a 200-triangle plane at
    -10 m/s with friction: plain FP64 bit for bit against the oracle."""
    sc = S.contact_cylinder(mu=(0.3, 0.2))
    o, g64 = ora(sc), gpu(sc)
    for d in (o, g64):
        d.step(300)
    for f in ("x", "u", "v", "pl_strain", "sigma_eq", "normal", "contforce"):
        assert np.array_equal(g64.get_field(f), o.get_field(f), equal_nan=True), f
    for f in ("ID", "cont_count"):
        assert np.array_equal(g64.get_field_i32(f), o.get_field_i32(f)), f
    assert (g64.get_field_i32("cont_count") > 0).sum() > 100


CONTACT_FIELDS = ("u", "pl_strain", "sigma_eq", "contforce")


def test_contact_mixed_within_1e3_frictionless():
    """Mixed form against plain FP64 under the frictionless plane: 1e-3."""
    sc = S.contact_cylinder(mu=(0.0, 0.0))
    g64, gm = gpu(sc), gpu(sc, {"precision": 1})
    for d in (g64, gm):
        d.step(300)
    for f in CONTACT_FIELDS:
        err = rel_l2(gm.get_field(f), g64.get_field(f))
        assert err < 1e-3, (f, err)
    Fz64, Fzm = g64.get_field("contforce")[:, 2].sum(), gm.get_field("contforce")[:, 2].sum()
    assert abs(Fzm - Fz64) <= 1e-3 * abs(Fz64)


def test_contact_mixed_with_friction_within_fp64_sensitivity():
    """With friction the stick/slip switch makes the problem ill-conditioned:
    two plain FP64 runs whose positions differ by 1e-12 (relative) already
    differ by ~5e-4 in u and ~5e-2 in the contact forces after 300 steps.  The
    mixed form must stay within three times that spread (and 1e-3)."""
    sc = S.contact_cylinder(mu=(0.3, 0.2))
    sp = dict(sc)
    sp["x"] = sc["x"] * (1.0 + 1e-12 * np.random.default_rng(3).standard_normal(sc["x"].shape))
    g64, gp, gm = gpu(sc), gpu(sp), gpu(sc, {"precision": 1})
    for d in (g64, gp, gm):
        d.step(300)
    for f in CONTACT_FIELDS:
        ref = g64.get_field(f)
        spread = rel_l2(gp.get_field(f), ref)
        err = rel_l2(gm.get_field(f), ref)
        assert err < max(1e-3, 3.0 * spread), (f, err, spread)


@pytest.mark.parametrize("case", ["beyond_edge", "behind_face", "face", "out_of_range",
                                  "slow_slide"])
def test_contact_law1_known_answers_gpu(case):
    """Contact law 1 for one particle under one triangle: the closed form, and
    the oracle bit for bit."""
    from weldformgpu_gb300 import Domain_d
    from tests.test_00_oracle import check_law1_closed_form, law1_one_step
    g, sc, exp = law1_one_step(Domain_d, case)
    check_law1_closed_form(g, sc, exp)
    o = law1_one_step(O.OracleDomain, case)[0]
    for f in ("x", "v", "contforce", "fric_heat", "dTdt"):
        assert np.array_equal(g.get_field(f), o.get_field(f)), f
    assert np.array_equal(g.get_field_i32("cont_count"), o.get_field_i32("cont_count"))


LAW1_FIELDS = ("x", "u", "v", "pl_strain", "sigma_eq", "contforce", "fric_heat")


def test_contact_law1_fp64_vs_oracle_with_adaptive_rebuild():
    """Block (12,288 particles) indented by a lower-half icosphere (656
    triangles) at -5 m/s: contact law 1 with friction and frictional heat, JC
    Newton, heat conduction, neighbour rebuild at a plastic-strain increment of
    0.002 (11 rebuilds in 600 steps).  Plain FP64 against the oracle: 1e-9
    (pow/log of JC and the heat terms may differ in the last bit), the same
    rebuild steps and the same contact set."""
    sc = S.indent_block(rebuild_increment=0.002)
    o, g = ora(sc), gpu(sc)
    for d in (o, g):
        d.step(600)
    nrb = g.get_scalar("rebuilds")
    assert nrb == o.get_scalar("rebuilds") and nrb >= 5
    for f in LAW1_FIELDS:
        err = rel_l2(g.get_field(f), o.get_field(f))
        assert err < 1e-9, (f, err)
    assert rel_l2(g.get_field("T") - 20.0, o.get_field("T") - 20.0) < 1e-9
    assert np.array_equal(g.get_field_i32("cont_count"), o.get_field_i32("cont_count"))
    assert (g.get_field_i32("cont_count") > 0).sum() >= 10
    assert g.get_field("T").max() > 30.0                 # frictional and plastic heating


def test_contact_law1_mixed_within_1e3():
    """Mixed form against plain FP64 on the icosphere indentation (law 1 is
    well conditioned: a 1e-12 relative change of the positions moves the
    contact forces by ~4e-9 after 300 steps): 1e-3 per field."""
    sc = S.indent_block(rebuild_increment=0.002)
    g64, gm = gpu(sc), gpu(sc, {"precision": 1})
    for d in (g64, gm):
        d.step(600)
    for f in ("u", "pl_strain", "sigma_eq", "contforce", "fric_heat"):
        err = rel_l2(gm.get_field(f), g64.get_field(f))
        assert err < 1e-3, (f, err)
    assert rel_l2(gm.get_field("T") - 20.0, g64.get_field("T") - 20.0) < 1e-3


def test_contact_law1_rejects_missing_dx():
    """Law 1 needs contact_dx: the solve fails with WF_ERR_STATE before any
    step and the domain is usable once it is set."""
    from weldformgpu_gb300 import Domain_d
    from weldformgpu_gb300.domain import WeldformError
    sc = S.indent_block(L=(0.002, 0.002, 0.001), R=0.002, level=2)
    opts = dict(sc["options"])
    del opts["contact_dx"]
    d = S.load(Domain_d(sc["n"]), dict(sc, options=opts))
    with pytest.raises(WeldformError) as e:
        d.step(1)
    assert e.value.code == -3 and "contact_dx" in str(e.value)
    d.set_option("contact_dx", sc["dx"])
    d.step(1)


def test_contact_law1_rotating_tool_fp64_vs_oracle_and_mixed():
    """A lower-half icosphere spinning at 2,000 rad/s about the z axis while it
    indents the centred block: its bins are rebuilt on the GPU every step, the
    friction and heat use the tool's surface velocity m_v + m_w x q.  Plain
    FP64 against the oracle's scan of every triangle: 1e-9 (pow/log) with the
    same contact set; the mixed form within 1e-3 of FP64."""
    sc = S.indent_block(rebuild_increment=0.002, omega=2000.0)
    o, g, gm = ora(sc), gpu(sc), gpu(sc, {"precision": 1})
    for d in (o, g, gm):
        d.step(600)
    for f in LAW1_FIELDS:
        err = rel_l2(g.get_field(f), o.get_field(f))
        assert err < 1e-9, (f, err)
    assert rel_l2(g.get_field("T") - 20.0, o.get_field("T") - 20.0) < 1e-9
    assert np.array_equal(g.get_field_i32("cont_count"), o.get_field_i32("cont_count"))
    cf = g.get_field("contforce")
    assert (g.get_field_i32("cont_count") > 0).sum() >= 10
    assert np.abs(cf[:, :2]).sum() > 0.2 * np.abs(cf[:, 2]).sum()   # the spin drags
    for f in ("u", "pl_strain", "contforce", "fric_heat"):
        err = rel_l2(gm.get_field(f), g.get_field(f))
        assert err < 1e-3, (f, err)


def test_set_positions_rejects_non_finite_and_keeps_state():
    """A NaN or infinite coordinate fails with WF_ERR_ARG before anything is
    written; valid positions then go in and read back unchanged."""
    from weldformgpu_gb300 import Domain_d
    from weldformgpu_gb300.domain import WeldformError
    sc = S.compression_cylinder()
    d = Domain_d(sc["n"])
    for bad in (np.nan, np.inf):
        x = sc["x"].copy()
        x[5, 1] = bad
        with pytest.raises(WeldformError) as e:
            d.set_positions(x.ravel())
        assert e.value.code == -1 and "non-finite" in str(e.value)
    d.set_positions(np.ascontiguousarray(sc["x"]).ravel())
    assert np.array_equal(d.get_field("x"), sc["x"])


def test_mixed_fused_integration_bit_identical_to_separate_pass():
    """Mixed form without contact: the integration fused into the acceleration
    pass (new positions to a second mirror) gives the separate integration
    pass's results bit for bit, through neighbour rebuilds and coupled heat."""
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    sc["k"], sc["cp"] = 167.0, 896.0
    opts = {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "precision": 1,
            "rebuild_every": 5, "rebuild_current_positions": 1, "rebuild_after_yield": 0}
    fused = gpu(sc, dict(opts, fuse_integrate=1))
    sep = gpu(sc, dict(opts, fuse_integrate=0))
    for n in (1, 7, 150):
        fused.step(n)
        sep.step(n)
        for f in ("x", "u", "v", "a", "rho", "pl_strain", "sigma_eq", "T"):
            assert np.array_equal(fused.get_field(f), sep.get_field(f)), (n, f)
    assert sep.get_field("pl_strain").max() > 0.0


@pytest.mark.parametrize("cap_max", [2048, 700])
def test_tile_staging_bit_identical_to_global_gathers(cap_max):
    """The mixed pair passes reading neighbours from per-tile halos in shared
    memory, and those reading 16-bit lists (offsets from each tile's base
    slot), give the same bits as the passes gathering through the 32-bit lists:
    JC with coupled heat and the tensor-core network, 300 steps with light
    rebuilds and a periodic reorder.  With tile_cap_max 700 part of the tiles
    exceed the halo capacity and gather from global memory inside the same
    launches."""
    from weldformgpu_gb300 import mlp
    sc = S.jc_compression(R=0.006, H=0.012)
    opts = {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "rebuild_every": 5,
            "rebuild_current_positions": 1, "rebuild_after_yield": 0, "precision": 1,
            "tile_cap_max": cap_max}
    runs = []
    for staging in (1, 0, 2):                    # 2: global gathers through 16-bit lists
        d = gpu(sc, dict(opts, tile_staging=1 if staging == 1 else 0, list16=int(staging == 2)))
        d.set_mlp_weights(mlp.init_params(3))
        d.set_option("mlp", 1)
        d.step(300)
        runs.append({f: d.get_field(f) for f in ("x", "v", "u", "shearstress", "pl_strain",
                                                 "sigma_eq", "T", "rho")})
        if staging == 1:
            tiles = (sc["n"] + 127) // 128
            staged = d.get_scalar("tiles_staged")
            hmax = d.get_scalar("tile_halo_max")
            if cap_max == 2048:
                assert staged == tiles, (staged, tiles)
            else:
                assert 0 < staged < tiles and hmax > cap_max, (staged, tiles, hmax)
        else:
            assert d.get_scalar("tile_cap") == 0
        d.close()
    for f in runs[0]:
        assert np.array_equal(runs[0][f], runs[1][f]), f
        assert np.array_equal(runs[2][f], runs[1][f]), f


@pytest.mark.parametrize("network", [0, 1])
def test_prefetch_options_do_not_change_results(network):
    """The L2 prefetches of the mixed passes (lists ahead, the tail's state,
    the next wave's prologue) are hints: every field is bit-identical with
    all of them off, with and without the tensor-core network (two stress
    kernels), including the call-end heat pass and the first-step density
    pass of each call."""
    from weldformgpu_gb300 import mlp
    sc = S.jc_compression(R=0.006, H=0.012)
    opts = {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "rebuild_every": 5,
            "rebuild_current_positions": 1, "rebuild_after_yield": 0, "precision": 1}
    runs = []
    for pf in ({}, {"list_prefetch": 0, "state_prefetch": 0, "wave_prefetch": 0},
               {"list_prefetch": 3, "wave_prefetch": 7, "wave_prefetch_distance": 0.5}):
        d = gpu(sc, dict(opts, **pf))
        if network:
            d.set_mlp_weights(mlp.init_params(3))
            d.set_option("mlp", 1)
        for n in (1, 37, 62):                    # calls: first-step density, call-end heat
            d.step(n)
        runs.append({f: d.get_field(f) for f in ("x", "v", "u", "shearstress", "pl_strain",
                                                 "sigma_eq", "T", "rho", "int_energy")})
        d.close()
    for f in runs[0]:
        assert np.array_equal(runs[0][f], runs[1][f]), f
        assert np.array_equal(runs[0][f], runs[2][f]), f


def test_mixed_fused_heat_matches_separate_heat_pass():
    """Mixed form: the heat pass fused into the next step's density pass gives
    the temperatures of the separate heat pass (to FP32 rounding), including
    across neighbour rebuilds, calls that end mid-run (the pending heat pass is
    run before results are read) and the first-step leapfrog."""
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    sc["k"], sc["cp"] = 167.0, 896.0
    opts = {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "precision": 1,
            "rebuild_every": 5, "rebuild_current_positions": 1, "rebuild_after_yield": 0}
    fused = gpu(sc, dict(opts, fuse_heat=1))
    sep = gpu(sc, dict(opts, fuse_heat=0))
    for n in (1, 7, 92):                       # uneven calls: flushes at odd places
        fused.step(n)
        sep.step(n)
        Tf, Ts = fused.get_field("T"), sep.get_field("T")
        assert rel_l2(Tf - 20.0, Ts - 20.0) < 1e-5
        assert rel_l2(fused.get_field("u"), sep.get_field("u")) < 1e-6
    assert Ts.max() > 20.5


@pytest.mark.parametrize("graph", [1, 0])
def test_timed_steps_with_per_launch_events(graph):
    """wf_time_steps with a kernel's launches timed by CUDA events: inside
    step graphs the events are event-record nodes, without graphs plain
    records; both report the launches and their time."""
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    d = gpu(sc, {"return_map": 1, "precision": 1, "graph": graph, "rebuild_after_yield": 0})
    d.step(3)
    d.set_option("profile_kernel", 2)        # the stress pass
    elapsed, kms, kl, total = d.time_steps(12)
    d.set_option("profile_kernel", 0)
    assert kl == 12 and 0.0 < kms < elapsed
    assert total >= 3 * 12
    assert (d.get_scalar("graph_launches") > 0) == bool(graph)


def test_setters_from_pinned_host_arrays_match_pageable():
    """The same scenario and checkpoint loaded from page-locked (pinned) and
    from pageable host arrays give identical fields, before and after steps
    (the end-to-end measurement passes pinned arrays)."""
    torch = pytest.importorskip("torch")
    from weldformgpu_gb300 import Domain_d
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    sc["k"], sc["cp"] = 167.0, 896.0
    opts = {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "precision": 1}
    keep = []

    def pinned(a):
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
        keep.append(t)
        out = t.numpy()
        out[...] = a
        return out

    base = gpu(sc, opts)
    base.step(40)
    state = base.checkpoint()
    psc = {k: (pinned(v) if isinstance(v, np.ndarray) else v) for k, v in sc.items()}
    pstate = {k: (pinned(v) if isinstance(v, np.ndarray) else v) for k, v in state.items()}
    a = S.load(Domain_d(sc["n"]), sc, opts)
    b = S.load(Domain_d(sc["n"]), psc, opts)
    a.restore(state)
    b.restore(pstate)
    fields = ("x", "u", "v", "rho", "pl_strain", "sigma_eq", "T")
    for f in fields:
        assert np.array_equal(a.get_field(f), b.get_field(f)), f
    a.step(30)
    b.step(30)
    for f in fields:
        assert np.array_equal(a.get_field(f), b.get_field(f)), f


def test_cached_arena_gives_a_fresh_domain():
    """wf_destroy keeps the arena for the next wf_create: a domain built on a
    reused arena (same size, and a smaller layout in the larger block) runs
    exactly as one built on fresh memory, after the old one was run hot."""
    from weldformgpu_gb300 import Domain_d, domain as D
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    opts = {"return_map": 1, "precision": 1, "energy_mode": 1}
    small = dict(sc)                     # the first 520 particles: a slightly smaller layout
    m = 520
    small.update(n=m, x=sc["x"][:m], m=sc["m"][:m], ids=sc["ids"][:m],
                 not_write=sc["not_write"][:m], T=sc["T"][:m])
    assert 0.9 * sc["n"] < m < sc["n"]
    fields = ("x", "u", "v", "rho", "sigma", "pl_strain", "sigma_eq", "int_energy")

    def run(scn):
        d = S.load(Domain_d(scn["n"]), scn, opts)
        d.step(60)
        out = {f: d.get_field(f) for f in fields}
        st = int(d.get_scalar("status"))
        d.close()
        return out, st

    assert D.lib().wf_release_cache() == 0
    fresh, st0 = run(sc)                 # on a fresh allocation
    again, st1 = run(sc)                 # on the arena the first run left
    assert D.lib().wf_release_cache() == 0
    fresh_small, _ = run(small)
    big, _ = run(sc)                     # leaves the larger block cached
    reused_small, _ = run(small)         # the smaller layout in it
    assert st0 == st1 == 0
    for f in fields:
        assert np.array_equal(fresh[f], again[f]), f
        assert np.array_equal(fresh[f], big[f]), f
        assert np.array_equal(fresh_small[f], reused_small[f]), f
    assert D.lib().wf_release_cache() == 0


def _graph_case(name):
    if name == "mixed_jc_heat":
        sc = S.compression_cylinder(material="jc", vz_top=-10.0)
        sc["k"], sc["cp"] = 167.0, 896.0
        return sc, {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "precision": 1,
                    "rebuild_every": 5, "rebuild_current_positions": 1, "rebuild_after_yield": 0}
    if name == "fp64_bilinear":   # status reads until the first yield, then rebuilds
        return S.compression_cylinder(), {}
    if name == "contact_law0_mixed":
        return S.contact_cylinder(mu=(0.3, 0.2)), {"precision": 1}
    if name == "mixed_jc_network":   # the tcgen05 warm start inside the stress pass
        sc = S.compression_cylinder(material="jc", vz_top=-10.0)
        return sc, {"return_map": 1, "precision": 1, "rebuild_after_yield": 0, "mlp": 1}
    # law 1, rotating tool (bins rebuilt on the GPU every step), periodic rebuilds
    return S.indent_block(rebuild_increment=0.0, omega=2000.0), {"precision": 1, "rebuild_every": 5}


@pytest.mark.parametrize("name", ["mixed_jc_heat", "fp64_bilinear", "contact_law0_mixed",
                                  "contact_law1_rotating_mixed", "mixed_jc_network"])
def test_step_graphs_bit_identical_to_direct_launches(name):
    """The steps between host synchronisation points replayed as one CUDA
    graph give the directly launched steps' results bit for bit, through
    uneven calls (segments cut at call ends) and neighbour rebuilds."""
    from weldformgpu_gb300 import Domain_d, mlp
    sc, opts = _graph_case(name)
    doms = []
    for g in (1, 0):
        d = Domain_d(sc["n"])
        if opts.get("mlp"):
            d.set_mlp_weights(mlp.init_params(3))   # untrained: starts accepted or rejected alike
        doms.append(S.load(d, sc, dict(opts, graph=g)))
    graph, direct = doms
    fields = ("x", "u", "v", "a", "rho", "pl_strain", "sigma_eq", "T")
    for n in (1, 7, 13, 123):
        graph.step(n)
        direct.step(n)
        for f in fields:
            assert np.array_equal(graph.get_field(f), direct.get_field(f)), (n, f)
    assert graph.get_scalar("graph_launches") > 0
    assert direct.get_scalar("graph_launches") == 0
    assert graph.get_scalar("rebuilds") == direct.get_scalar("rebuilds")


def test_reference_api_mech_fraser_solve_bit_exact():
    """MechFraserSolve(tf, dt_out) through the reference's method names: stale
    (last-output) positions for the rebuilds, outputs every dt_out."""
    from weldformgpu_gb300 import Domain_d
    sc = S.compression_cylinder()
    d = Domain_d(sc["n"])
    d.Set_h(sc["h"])
    d.SetDensity(sc["rho"])
    d.SetShearModulus(sc["G"])
    d.SetSigmay(sc["sy"])
    d.SetCs(np.full(sc["n"], sc["Cs"]))
    d.SetFreePart(np.ones(sc["n"], np.uint8))
    d.SetID(sc["ids"])
    d.set_positions(sc["x"])
    d.set_mass(sc["m"])
    d.set_time_step(sc["dt"])
    d.set_material(sc["mat"])
    for z, v in sc["bcs"]:
        d.add_velocity_bc(z, *v)
    tf, dt_out = 700 * sc["dt"], 64 * sc["dt"]
    d.MechFraserSolve(tf, dt_out)
    o = ora(sc)
    o.mech_fraser_solve(tf, dt_out)
    for f in ("x", "v", "sigma", "pl_strain"):
        assert np.array_equal(d.get_field(f), o.get_field(f)), f


def test_write_csv_reference_columns(tmp_path):
    sc = S.compression_cylinder()
    g = gpu(sc)
    g.step(3)
    path = tmp_path / "out.csv"
    g.WriteCSV(str(path))
    lines = path.read_text().splitlines()
    assert lines[0].startswith("ID, X, Y, Z, posX,posY,posZ,Ux, Uy, Uz")
    assert len(lines) == sc["n"] + 1
    assert len(lines[1].split(",")) == 29


def test_release_cache_returns_the_arena_to_the_driver():
    """wf_destroy keeps the arena cached (device memory stays allocated) and
    wf_release_cache frees it: the free device memory returns to its level
    before the domain was created."""
    torch = pytest.importorskip("torch")
    from weldformgpu_gb300 import Domain_d, domain as D
    sc = S.jc_compression(R=0.012, H=0.024)          # ~0.1M particles, an arena of ~140 MB
    assert D.lib().wf_release_cache() == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    d = S.load(Domain_d(sc["n"]), sc, {"precision": 1})
    d.step(2)
    d.close()
    torch.cuda.synchronize()
    free_cached = torch.cuda.mem_get_info()[0]
    assert D.lib().wf_release_cache() == 0
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free_cached > 64 << 20                  # the arena is still held
    assert abs(free1 - free0) < 32 << 20, (free0, free_cached, free1)


def test_debug_checks_repair_and_report_an_injected_list_error():
    """Option debug_checks (the stand-in for a bounds-checking sanitizer):
    with nothing wrong it changes no bit of the results; a list entry set out
    of range on the device (host-side injection, between the list build and
    the check) is repaired before any pass reads it, reported in status bit 6
    and by the call's return code, and leaves the state finite.  The injection
    is refused without the checks."""
    from weldformgpu_gb300.domain import WeldformError
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    opts = {"return_map": 1, "precision": 1}
    ref = gpu(sc, opts)
    ref.step(30)
    a = gpu(sc, dict(opts, debug_checks=1))
    a.step(30)
    for f in ("x", "v", "u", "sigma_eq", "pl_strain"):
        assert np.array_equal(a.get_field(f), ref.get_field(f)), f
    assert int(a.get_scalar("status")) & 64 == 0
    b = gpu(sc, opts)
    with pytest.raises(WeldformError):
        b.set_option("debug_inject_list_error", 100)
    c = gpu(sc, dict(opts, debug_checks=1))
    c.set_option("debug_inject_list_error", 100)
    with pytest.raises(WeldformError):
        c.step(30)
    assert int(c.get_scalar("status")) & 64
    for f in ("x", "v", "sigma_eq"):
        assert np.all(np.isfinite(c.get_field(f))), f
