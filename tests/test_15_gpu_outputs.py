"""GPU: the FP64 output reductions, Newton-cap reporting, the per-step host
hook and position restores, through the C ABI.

Tolerances:
  - maxima of bit-exact fields (plain FP64 form): equal;
  - FP64 sums (BC reactions, contact force sums, energy): the GPU reduces in a
    fixed tree order, the oracle sequentially, so they agree to
    1e-12 of the sum of the magnitudes of their terms;
  - mixed form: reaction curve within 1e-3 relative L2 of the plain FP64 run.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import scenarios as S

pytestmark = pytest.mark.gpu


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


def assert_rows_match(rg, ro, n_terms):
    """time, step and maxima equal; every sum within 1e-12 of the oracle's
    largest value of that column times the number of its terms."""
    assert rg.shape == ro.shape, (rg.shape, ro.shape)
    np.testing.assert_array_equal(rg[:, :2], ro[:, :2])            # time, step
    np.testing.assert_array_equal(rg[:, 2:6], ro[:, 2:6])          # maxima of bit-exact fields
    for k in range(6, rg.shape[1]):
        if k >= 11:    # a BC's three components share the scale of its largest one
            b = (k - 11) // 3
            scale = np.abs(ro[:, 11 + 3 * b:14 + 3 * b]).max()
        else:
            scale = np.abs(ro[:, k]).max()
        tol = 1e-12 * scale * n_terms[k]
        err = np.max(np.abs(rg[:, k] - ro[:, k]))
        assert err <= tol, (k, err, tol)


def test_output_rows_fp64_vs_oracle_compression():
    """Bilinear compression (R 5 mm, H 10 mm cylinder, 400 steps): every-step rows;
    the top platen's reaction grows as the cylinder is loaded."""
    sc = S.compression_cylinder(R=0.005, H=0.010)
    opts = {"output_every_step": 1}
    g, o = gpu(sc, opts), ora(sc, opts)
    g.step(400)
    o.step(400)
    rg, ro = g.get_output_series(), o.get_output_series()
    assert rg.shape == (400, 11 + 3 * 2)
    n = sc["n"]
    zones = [int((sc["ids"] == z).sum()) for z, _ in sc["bcs"]]
    assert_rows_match(rg, ro, [n] * 11 + [zones[0]] * 3 + [zones[1]] * 3)
    fz_top = rg[:, 11 + 3 * 1 + 2]
    assert fz_top[-1] > 0.0 and abs(fz_top[-1]) > 10 * abs(fz_top[10])   # loading up
    np.testing.assert_array_equal(g.get_reaction(1), rg[-1, 14:17])
    assert g.get_scalar("reaction_z") == rg[-1, 13]                      # BC 0
    assert g.get_scalar("max_pl_strain") == rg[-1, 5]


def test_output_rows_at_output_times_and_csv(tmp_path):
    """Without output_every_step, MechFraserSolve records a row per output
    time and writes them to <prefix>outputs.csv; the values equal the
    every-step series at those steps."""
    sc = S.compression_cylinder(R=0.005, H=0.010)
    dt = sc["dt"]
    a = gpu(sc)
    b = gpu(sc, {"output_every_step": 1})
    a.set_csv_output(str(tmp_path) + "/")
    a.mech_fraser_solve(120 * dt, 40 * dt)
    b.mech_fraser_solve(120 * dt, 40 * dt)
    ra, rb = a.get_output_series(), b.get_output_series()
    assert len(ra) >= 3
    for r in ra:
        k = np.where(rb[:, 1] == r[1])[0]
        assert len(k) == 1
        np.testing.assert_array_equal(r, rb[k[0]])
    lines = (tmp_path / "outputs.csv").read_text().strip().splitlines()
    assert lines[0].startswith("time, step, max_ux") and len(lines) == len(ra) + 1


def test_output_rows_contact_force_sum_vs_oracle():
    """The reference's contact force sum (|contforce| over free-surface
    particles) under the rigid plane with friction, FP64 vs the oracle."""
    sc = S.contact_cylinder(mu=(0.3, 0.2))
    opts = {"output_every_step": 1}
    g, o = gpu(sc, opts), ora(sc, opts)
    g.step(300)
    o.step(300)
    rg, ro = g.get_output_series(), o.get_output_series()
    assert ro[-1, 6] > 0.0
    n = sc["n"]
    zones = [int((sc["ids"] == z).sum()) for z, _ in sc["bcs"]]
    assert_rows_match(rg, ro, [n] * 11 + [zones[0]] * 3 + [zones[1]] * 3)


def test_mixed_reaction_curve_within_1e3_of_fp64():
    """JC compression with heat, mixed form vs plain FP64 of the same code:
    the top platen's reaction curve (every step) within 1e-3 relative L2."""
    sc = S.compression_cylinder(R=0.004, H=0.008, material="jc", vz_top=-10.0,
                                generator="lattice", dt_rule="sound_speed")
    sc["k"], sc["cp"] = 167.0, 896.0
    opts = {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "output_every_step": 1,
            "rebuild_every": 10, "rebuild_current_positions": 1, "rebuild_after_yield": 0}
    a = gpu(sc, dict(opts, precision=0))
    b = gpu(sc, dict(opts, precision=1))
    a.step(600)
    b.step(600)
    ra, rb = a.get_output_series(), b.get_output_series()
    fa, fb = ra[:, 11 + 3 + 2], rb[:, 11 + 3 + 2]
    assert np.abs(fa).max() > 0.0
    assert rel_l2(fb, fa) <= 1e-3, rel_l2(fb, fa)


def test_newton_cap_is_reported():
    """newton_max_iter = 1 on a plastic JC case: the return maps stop before
    the tolerance, the counter and status bit are set and the call returns
    WF_ERR_NUMERIC; with the default cap none stops early."""
    from weldformgpu_gb300.domain import WeldformError
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    for precision in (0, 1):
        d = gpu(sc, {"return_map": 1, "precision": precision, "newton_max_iter": 1})
        with pytest.raises(WeldformError) as e:
            d.step(300)
        assert e.value.code == -5 and "newton_max_iter" in str(e.value)
        assert d.get_scalar("newton_capped") > 0
        assert int(d.get_scalar("status")) & 16
        ok = gpu(sc, {"return_map": 1, "precision": precision})
        ok.step(300)
        assert ok.get_scalar("newton_calls") > 0
        assert ok.get_scalar("newton_capped") == 0
    o = ora(sc, {"return_map": 1, "newton_max_iter": 1})
    o.step(300)
    assert o.get_scalar("newton_capped") > 0
    from weldformgpu_gb300.domain import Domain_d
    d = Domain_d(4)
    with pytest.raises(WeldformError):
        d.set_option("newton_max_iter", 0)


def test_step_callback_ramp_matches_oracle_stepped_by_hand():
    """The GeneralAfter hook: a callback ramps the top BC's velocity with time
    inside one wf_step call; the oracle, stepped one step at a time with the
    same velocity set between steps, gives the same state bit for bit.  An
    identity callback leaves the run bit-identical to one without."""
    sc = S.compression_cylinder(R=0.005, H=0.010)
    t_ramp = 150 * sc["dt"]

    def v_of(t):
        return -2.0 * min(t / t_ramp, 1.0)

    g = gpu(sc)
    calls = []

    def hook(dom):
        t = dom.get_scalar("time")
        calls.append(t)
        dom.set_velocity_bc(1, 0.0, 0.0, v_of(t))
        return 0
    g.set_velocity_bc(1, 0.0, 0.0, v_of(0.0))
    g.set_callback(hook)
    g.step(300)
    o = ora(sc)
    o.set_velocity_bc(1, 0.0, 0.0, v_of(0.0))
    for _ in range(300):
        o.step(1)
        o.set_velocity_bc(1, 0.0, 0.0, v_of(o.get_scalar("time")))
    assert len(calls) == 300
    for f in ("x", "u", "v", "sigma", "pl_strain"):
        assert np.array_equal(g.get_field(f), o.get_field(f)), f
    # identity hook vs none (graphs on in the second)
    a, b = gpu(sc), gpu(sc)
    a.set_callback(lambda dom: 0)
    a.step(120)
    b.step(120)
    for f in ("x", "v", "sigma"):
        assert np.array_equal(a.get_field(f), b.get_field(f)), f
    # a non-zero return ends the solve; solvers cannot be called from the hook
    from weldformgpu_gb300.domain import WeldformError
    c = gpu(sc)
    c.set_callback(lambda dom: 7)
    with pytest.raises(WeldformError) as e:
        c.step(5)
    assert e.value.code == -3 and "returned 7" in str(e.value)
    assert c.get_scalar("step") == 1
    seen = []

    def reenter(dom):
        try:
            dom.step(1)
        except WeldformError as err:
            seen.append(err.code)
        return 0
    c.set_callback(reenter)
    c.step(2)
    assert seen == [-3, -3]


def test_restored_positions_rebuild_lists_and_reject_non_finite():
    """wf_set_field("x") mid-run goes through the finite check and makes the
    next step rebuild the lists for the restored positions: restoring a
    checkpoint into a running domain continues exactly like restoring it into
    a fresh one (whose solve start builds the lists)."""
    from weldformgpu_gb300.domain import WeldformError
    sc = S.compression_cylinder(R=0.004, H=0.008)
    sc["options"] = {"rebuild_every": 1000, "rebuild_after_yield": 0}
    base = gpu(sc)
    base.step(100)
    st = base.checkpoint()
    runner = gpu(sc)
    runner.step(37)                         # its lists belong to other positions
    bad = st["x"].copy()
    bad[1234 % sc["n"], 1] = np.nan
    with pytest.raises(WeldformError) as e:
        runner.set_field("x", bad)
    assert e.value.code == -1
    runner.restore(st)
    fresh = gpu(sc)
    fresh.restore(st)
    runner.step(50)
    fresh.step(50)
    for f in ("x", "v", "sigma", "pl_strain"):
        assert np.array_equal(runner.get_field(f), fresh.get_field(f)), f
