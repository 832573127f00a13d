"""The oracle against the reference: golden vectors (CPU, every machine) and,
where the reference tree is present, the reference's kernels run live.

The oracle restates the reference's arithmetic in the reference's operation
order, so the comparisons are exact (np.array_equal), not tolerances.
"""
import os

import numpy as np
import pytest

from oracle import build_ref, oracle as O
from tests import scenarios as S
from weldformgpu_gb300 import _abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STATE_FIELDS = ["x", "v", "a", "rho", "drho", "p", "sigma", "shearstress", "strrate", "rotrate",
                "sigma_eq", "pl_strain", "sigma_y", "eff_strain_rate", "int_energy"]


def _oracle(sc, options=None):
    return S.load(O.OracleDomain(sc["n"]), sc, options)


def test_neighbors_small_match_reference_cunsearch():
    g = np.load(os.path.join(GOLDEN, "nb_small.npz"))
    d = O.OracleDomain(len(g["x"]))
    d.set_h(float(g["h"]))
    d.set_positions(g["x"].ravel())
    d.find_neighbors()
    cnt, lst = d.get_neighbors()
    assert np.array_equal(cnt, g["counts"])
    for i in range(len(cnt)):
        # same set AND same order: sequential cuNSearch fills cells in index order
        assert np.array_equal(lst[i, :cnt[i]], g["lists"][i, :cnt[i]])


def test_neighbour_rule_at_the_support_radius_matches_float32():
    """Pairs within ~3 float32 ulps of r = 2h: the oracle's lists are those of
    the float rule evaluated with numpy float32 (rounded differences, squares
    and sum, no fused multiply-add; d^2 < r^2), about half the pairs in."""
    h = 1.0e-3
    x = S.support_radius_pairs(h)
    n = len(x)
    d = O.OracleDomain(n)
    d.set_h(h)
    d.set_positions(np.ascontiguousarray(x).ravel())
    d.find_neighbors()
    cnt, lst = d.get_neighbors()
    xf = x.astype(np.float32)
    dd = xf[1::2] - xf[0::2]
    s = (dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1]) + dd[:, 2] * dd[:, 2]
    r = np.float32(2.0 * h)
    inside = s < r * r
    assert s.dtype == np.float32
    assert np.array_equal(cnt[0::2] == 1, inside) and np.array_equal(cnt[1::2] == 1, inside)
    assert np.array_equal(lst[0::2, 0][inside], np.arange(1, n, 2)[inside])
    assert 0.3 < inside.mean() < 0.7


def test_neighbors_cylinder_r5mm_digest():
    g = np.load(os.path.join(GOLDEN, "nb_c1.npz"))
    c1 = S.compression_cylinder(R=0.005, H=0.010)
    assert c1["n"] == int(g["n"]) == 5244          # reference generator count
    d = O.OracleDomain(c1["n"])
    d.set_h(c1["h"])
    d.set_positions(c1["x"].ravel())
    d.find_neighbors()
    cnt, lst = d.get_neighbors()
    assert np.array_equal(cnt, g["counts"])
    from tests.golden.make_golden import list_digest
    s1, s2, dig = list_digest(cnt, lst)
    assert np.array_equal(s1, g["sum"]) and np.array_equal(s2, g["sumsq"])
    assert dig == str(g["sha256"])
    # every particle sees at most the reference cap, interior particles 56
    assert cnt.max() == 56 and cnt.max() <= _abi.WF_MAX_NEIGHBORS


@pytest.mark.parametrize("case,checkpoints", [("bilinear", [1, 600, 1500]), ("jc", [300]),
                                              ("hollomon", [300])])
def test_fraser_loop_matches_reference_bitwise(case, checkpoints):
    g = np.load(os.path.join(GOLDEN, "fraser_%s.npz" % case))
    sc = (S.compression_cylinder() if case == "bilinear"
          else S.compression_cylinder(material=case, vz_top=-10.0))
    d = _oracle(sc)
    done = 0
    for k in checkpoints:
        d.step(k - done)
        done = k
        for f in STATE_FIELDS:
            ref = g["s%d_%s" % (k, f)]
            got = d.get_field(f)
            assert np.array_equal(got, ref), "%s step %d field %s differs (max |d| %.3e)" % (
                case, k, f, np.max(np.abs(got - ref)))
    if case == "bilinear":
        assert d.get_field("pl_strain").max() > 0.05      # plastic, rebuilt lists
        assert d.get_scalar("is_yielding") == 1.0


def test_generators_match_between_oracle_and_library():
    from weldformgpu_gb300 import setup as P
    x1, m1 = P.gen_cylinder_ref((0.0, 0.0, -0.028), 0.15, 0.616, 0.0075, 2700.0)
    x2, m2 = O.gen_cylinder_ref((0.0, 0.0, -0.028), 0.15, 0.616, 0.0075, 2700.0)
    assert len(x1) == 11316                    # examples/input/Compression.json
    assert np.array_equal(x1, x2) and m1 == m2
    b1, bm1 = P.gen_box_cubic((0, 0, 0), (1e-3, 2e-3, 1.5e-3), 5e-5, 7850.0)
    b2, bm2 = O.gen_box_cubic((0, 0, 0), (1e-3, 2e-3, 1.5e-3), 5e-5, 7850.0)
    assert np.array_equal(b1, b2) and bm1 == bm2 and len(b1) == 10 * 20 * 15
    l1 = P.gen_cylinder_lattice(0.005, 0.010, 0.0005, 0.01, 1)
    l2 = O.gen_cylinder_lattice(0.005, 0.010, 0.0005, 0.01, 1)
    assert np.array_equal(l1, l2)
    assert 6000 < len(l1) < 6600                # R 5 mm, H 10 mm lattice: ~6.3k particles
    ids1 = np.zeros(len(l1), np.int32)
    ids2 = np.zeros(len(l1), np.int32)
    nw1 = np.zeros(len(l1), np.uint8)
    nw2 = np.zeros(len(l1), np.uint8)
    c1 = P.assign_zone(l1, (-1, -1, -1), (1, 1, 0.001), 2, ids1, nw1)
    c2 = O.assign_zone(l2, (-1, -1, -1), (1, 1, 0.001), 2, ids2, nw2)
    assert c1 == c2 > 0 and np.array_equal(ids1, ids2) and np.array_equal(nw1, nw2)
    # the "Cylindrical" grid: full cylinder and a pi/16 slice with its side ids
    for ang, rows, ri in ((2.0 * np.pi, 1, 0.0), (np.pi / 16.0, 1, 0.0025)):
        u1 = P.gen_cylinder_uniform(0.005, 0.004, 0.00025, 2700.0, ang, rows, ri)
        u2 = O.gen_cylinder_uniform(0.005, 0.004, 0.00025, 2700.0, ang, rows, ri)
        assert np.array_equal(u1[0], u2[0]) and np.array_equal(u1[1], u2[1]) and u1[2] == u2[2]
        n = len(u1[0])
        assert u1[2] == np.pi * 0.005 * 0.005 * 0.004 * 2700.0 / n    # Domain.cpp:1171-1173
        assert np.allclose(np.unique(np.round(u1[0][:, 2] / 0.00025)), np.arange(1, 16, 2))
        if ang < 2.0 * np.pi:
            assert {2, 3} <= set(u1[1].tolist())
        else:
            assert set(u1[1].tolist()) == {0, 4} and (u1[1] == 4).sum() == 8   # axis
    for positive in (0, 1):
        m1 = P.gen_plane_mesh(2, positive, (-0.003, -0.003, 0.006), (0.003, 0.003, 0.006), 7)
        m2 = O.gen_plane_mesh(2, positive, (-0.003, -0.003, 0.006), (0.003, 0.003, 0.006), 7)
        assert all(np.array_equal(a, b) for a, b in zip(m1, m2))
        assert m1[0].shape == (64, 3) and m1[1].shape == (98, 3)


def test_contact_matches_reference_bitwise():
    """A rigid plane pressing the small cylinder (surface tagging, contact
    lists, the penalty law with friction, mesh motion, rigid particles), against
    the reference's own contact kernels: every field and the ids bit for bit."""
    g = np.load(os.path.join(GOLDEN, "fraser_contact.npz"))
    sc = S.contact_cylinder(R=0.0025, H=0.005, dens=6, mu=(0.3, 0.2))
    d = _oracle(sc)
    done = 0
    for k in (1, 200, 600):
        d.step(k - done)
        done = k
        for f in STATE_FIELDS + ["u", "normal", "contforce"]:
            ref = g["s%d_%s" % (k, f)]
            got = d.get_field(f)
            assert np.array_equal(got, ref, equal_nan=True), "step %d field %s differs" % (k, f)
        assert np.array_equal(d.get_field_i32("ID"), g["s%d_ID" % k])
    assert (np.abs(d.get_field("contforce")).sum(axis=1) > 0).sum() > 20     # in contact
    assert d.get_field("pl_strain").max() > 0.1


# Contact law 1 known answers: one particle and one triangle (normal -z at
# z = 4e-4, dx = 1e-3, contact radius dx/2): x0, the tool velocity and the
# nearest point on the triangle.
TRI = [(-0.01, -0.01, 4e-4), (-0.01, 0.01, 4e-4), (0.01, -0.01, 4e-4)]
LAW1_CASES = {
    "face": ((-0.002, -0.002, 0.0), (-2.0, 0.0, -5.0), (-0.002, -0.002, 4e-4)),
    "beyond_edge": ((-0.0102, 0.0, 1e-4), (-2.0, -1.0, -5.0), (-0.01, 0.0, 4e-4)),
    "slow_slide": ((-0.002, -0.002, 0.0), (0.0, -4e-4, 0.0), (-0.002, -0.002, 4e-4)),
    "behind_face": ((-0.002, -0.002, 5e-4), (-1.0, 0.0, -5.0), (-0.002, -0.002, 4e-4)),
    "out_of_range": ((-0.002, -0.002, -2e-4), (-2.0, 0.0, -5.0), (-0.002, -0.002, 4e-4)),
}


def law1_one_step(make_domain, case):
    x0, v_tool, q = LAW1_CASES[case]
    sc, expected = S.one_particle_under_triangle(x0, TRI, v_tool)
    d = S.load(make_domain(sc["n"]), sc)
    d.step(1)
    return d, sc, expected(q)


def check_law1_closed_form(d, sc, exp):
    f, qf, n = exp
    m, dt = sc["m"][0], sc["dt"]
    got = d.get_field("contforce")[0]
    np.testing.assert_allclose(got, f, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(f).max()))
    np.testing.assert_allclose(d.get_field("fric_heat")[0], qf, rtol=1e-12, atol=1e-300)
    assert d.get_field_i32("cont_count")[0] == (1 if np.abs(f).max() > 0 else 0)
    np.testing.assert_allclose(d.get_field("v")[0], f / m * dt, rtol=1e-14, atol=1e-300)
    np.testing.assert_allclose(d.get_field("dTdt")[0], qf / (m * 896.0), rtol=1e-12,
                               atol=1e-300)


@pytest.mark.parametrize("case", sorted(LAW1_CASES))
def test_contact_law1_known_answers(case):
    """Penalty 0.1 K dx delta along the nearest-point normal (the face normal
    for a centre behind the face), regularised Coulomb friction and its heat,
    against the closed form for one particle under one triangle."""
    d, sc, exp = law1_one_step(O.OracleDomain, case)
    check_law1_closed_form(d, sc, exp)
    f, qf, n = exp
    if case == "beyond_edge":
        assert abs(n[2]) < 0.9 and abs(n[0]) > 0.5           # the edge normal, not the face's
    if case == "out_of_range":
        assert not f.any() and qf == 0.0
    else:
        assert np.abs(f).max() > 0.0 and qf > 0.0


# ---- analytic known answers of the SPH discretisation --------------------
DX, H_DX = 1.0e-3, 1.2


def lattice_moment():
    """kappa with sum_j V_j GK_ij x_ij x_ij^T = -kappa I on the cubic lattice
    at h = 1.2 dx (exactly -I for the continuous kernel)."""
    L = O.lib()
    g = np.arange(-3, 4)
    X = np.array(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1).T * DX
    X = X[np.any(X != 0, axis=1)]
    h = H_DX * DX
    GK = np.array([L.wfo_grad_kernel(q, h) for q in np.linalg.norm(X, axis=1) / h])
    M = (DX ** 3 * GK[:, None, None] * X[:, :, None] * X[:, None, :]).sum(0)
    assert np.abs(M - M[0, 0] * np.eye(3)).max() < 1e-12       # isotropic
    return -M[0, 0]


def elastic_box(dims, rho=2700.0, E=70e9, nu=0.33, ids=None):
    x, m = O.gen_box_cubic((0.0, 0.0, 0.0), tuple(k * DX for k in dims), DX / 2, rho)
    n = len(x)
    K, G = E / (3 * (1 - 2 * nu)), E / (2 * (1 + nu))
    Cs = np.sqrt(K / rho)
    h = H_DX * DX
    d = O.OracleDomain(n)
    d.set_h(h)
    d.set_density(rho)
    d.set_shear_modulus(G)
    d.set_sigma_y(1e12)
    d.set_cs(np.full(n, Cs))
    d.set_positions(x.ravel())
    d.set_mass(np.full(n, m))
    d.set_id(np.zeros(n, np.int32) if ids is None else ids(x))
    d.set_not_write_surf_id(np.zeros(n, np.uint8))
    d.set_time_step(0.4 * h / Cs)
    d.set_artificial_viscosity(1.0, 0.0)
    d.set_material(_abi.WfMaterial(model=_abi.WF_BILINEAR, E=E, nu=nu, sy0=1e12, Et=0.0))
    d.set_temperature(np.full(n, 20.0))
    return d, x, dict(K=K, G=G, rho=rho, E=E, dt=0.4 * h / Cs)


def interior(x, margin):
    c = 0.5 * (x.min(axis=0) + x.max(axis=0))
    half = 0.5 * (x.max(axis=0) - x.min(axis=0))
    return np.all(np.abs(x - c) <= half - margin, axis=1)


def test_kernel_gradient_moment_is_minus_three():
    """int grad W . x dV = -3 int W dV = -3 for the oracle's GradKernel (cubic
    spline, Functions.cu:76-88), by quadrature over the support; and the
    lattice moment at h = 1.2 dx is within 2 % of the continuous one."""
    from scipy.integrate import quad
    L = O.lib()
    for h in (1.0, 1.2e-3):
        f = lambda r: 4.0 * np.pi * r ** 4 * L.wfo_grad_kernel(r / h, h)   # noqa: E731
        val = quad(f, 0.0, h, epsabs=0, epsrel=1e-13)[0] + quad(f, h, 2 * h, epsabs=0,
                                                                 epsrel=1e-13)[0]
        assert abs(val + 3.0) < 1e-10, (h, val)
    assert abs(lattice_moment() - 1.0) < 0.02


def test_linear_velocity_field_rates_and_density_on_lattice():
    """v = L x on a cubic lattice: interior strain rate kappa sym(L), rotation
    rate kappa/2 (L - L^T) with the reference's sign flip of the xz entry
    (InteractionAlt.cu:362), density rate -kappa rho tr(L) (continuity)."""
    kappa = lattice_moment()
    d, x, p = elastic_box((12, 12, 12))
    Lg = np.array([[1.0, 0.3, -0.2], [0.5, -0.7, 0.4], [0.1, 0.6, 0.2]]) * 100.0
    d.set_velocities(np.ascontiguousarray(x @ Lg.T).ravel())
    d.find_neighbors()
    d.run_stage("density")
    d.run_stage("rates")
    inner = interior(x, 2.5 * DX)
    assert inner.sum() == 216
    S = 0.5 * (Lg + Lg.T) * kappa
    exp_sr = [S[0, 0], S[1, 1], S[2, 2], S[0, 1], S[1, 2], S[0, 2]]
    W = 0.5 * kappa * (Lg - Lg.T)
    exp_rr = [0.0, 0.0, 0.0, W[0, 1], W[1, 2], -W[0, 2]]
    np.testing.assert_allclose(d.get_field("strrate")[inner], np.tile(exp_sr, (216, 1)),
                               rtol=1e-10, atol=1e-10 * np.abs(exp_sr).max())
    np.testing.assert_allclose(d.get_field("rotrate")[inner], np.tile(exp_rr, (216, 1)),
                               rtol=1e-10, atol=1e-10 * np.abs(exp_rr).max())
    np.testing.assert_allclose(d.get_field("drho")[inner], -kappa * p["rho"] * np.trace(Lg),
                               rtol=1e-10)


def test_uniaxial_strain_rate_gives_p_wave_modulus():
    """One stress update under v = (e x, 0, 0): sigma_xx = (K + 4G/3) kappa e dt,
    sigma_yy = sigma_zz = (K - 2G/3) kappa e dt (EOS pressure from the density
    increment, deviatoric Hooke increment; rates see the updated density)."""
    kappa = lattice_moment()
    d, x, p = elastic_box((12, 12, 12))
    e = -100.0
    v = np.zeros_like(x)
    v[:, 0] = e * x[:, 0]
    d.set_velocities(v.ravel())
    d.find_neighbors()
    for stage in ("density", "update_density", "rates", "pressure", "stress"):
        d.run_stage(stage)
    # neighbours whose own neighbourhoods are complete (their density exact)
    inner = interior(x, 4.0 * DX)
    assert inner.sum() == 64
    K, G, dt = p["K"], p["G"], p["dt"]
    de = kappa * e * dt
    vol = 1.0 / (1.0 - de)                       # V_j = m / rho_new
    sg = d.get_field("sigma")[inner]
    np.testing.assert_allclose(sg[:, 0], K * de + 4.0 / 3.0 * G * de * vol, rtol=1e-9)
    np.testing.assert_allclose(sg[:, 1], K * de - 2.0 / 3.0 * G * de * vol, rtol=1e-9)
    np.testing.assert_allclose(sg[:, 2], K * de - 2.0 / 3.0 * G * de * vol, rtol=1e-9)
    assert np.abs(sg[:, 3:]).max() < 1e-9 * abs(sg[:, 0]).max()


def test_elastic_wave_front_speed():
    """A face pushed at 1 m/s into an elastic block (28 x 28 cross-section):
    the half-amplitude front on the centre line, before the lateral release
    waves reach it, travels at the longitudinal speed sqrt((K + 4G/3)/rho)
    within 5 % (the bar speed sqrt(E/rho) is 18 % lower)."""
    O.set_threads(os.cpu_count() or 1)
    d, x, p = elastic_box((40, 28, 28), ids=lambda x: np.where(x[:, 0] < 2 * DX, 2, 0).astype(
        np.int32))
    d.add_velocity_bc(2, 1.0, 0.0, 0.0)
    cL = np.sqrt((p["K"] + 4.0 * p["G"] / 3.0) / p["rho"])
    c = 0.5 * (x.min(axis=0) + x.max(axis=0))
    line = (np.abs(x[:, 1] - c[1]) < 0.6 * DX) & (np.abs(x[:, 2] - c[2]) < 0.6 * DX)
    order = np.argsort(x[line, 0])
    xl = x[line, 0][order]
    t, f = [], []
    d.step(6)
    for _ in range(8):
        d.step(2)
        vx = d.get_field("v")[line, 0][order]
        k = np.nonzero(vx >= 0.5)[0].max()
        t.append(d.get_scalar("time"))
        f.append(xl[k] + (vx[k] - 0.5) / (vx[k] - vx[k + 1]) * DX)
    speed = np.polyfit(t, f, 1)[0]
    assert abs(speed / cL - 1.0) < 0.05, (speed, cL)
    assert speed > 1.1 * np.sqrt(p["E"] / p["rho"])


def test_heat_conduction_step_matches_erfc():
    """Heat-only solve (ThermalSolve) of a temperature step in a steel bar
    (48 x 12 x 12 dx): along the centre line the profile follows
    T0 + (T1 - T0)/2 erfc((x - xm)/(2 sqrt(kappa alpha t))) within 1.5 % of the
    step after 100 steps (diffusion length 3 dx)."""
    from scipy.special import erfc
    kappa = lattice_moment()
    rho, cp, k = 7850.0, 460.0, 50.0
    alpha = k / (rho * cp)
    x, m = O.gen_box_cubic((0.0, 0.0, 0.0), (48 * DX, 12 * DX, 12 * DX), DX / 2, rho)
    n = len(x)
    xm, T0, T1 = 24 * DX, 20.0, 120.0
    dt = 0.1 * DX * DX / alpha
    d = O.OracleDomain(n)
    d.set_h(H_DX * DX)
    d.set_density(rho)
    d.set_positions(x.ravel())
    d.set_mass(np.full(n, m))
    d.set_conductivity(k)
    d.set_heat_cap(cp)
    d.set_temperature(np.where(x[:, 0] < xm, T1, T0))
    d.set_thermal_bc(np.zeros(n, np.int32))
    d.set_convection(0.0, T0)
    d.set_time_step(dt)
    d.thermal_solve(100 * dt * (1.0 - 1e-9))
    assert d.get_scalar("step") == 100
    t = d.get_scalar("time")
    c = 0.5 * (x.min(axis=0) + x.max(axis=0))
    line = (np.abs(x[:, 1] - c[1]) < 0.6 * DX) & (np.abs(x[:, 2] - c[2]) < 0.6 * DX)
    mid = line & (np.abs(x[:, 0] - xm) < 12 * DX)
    exact = T0 + 0.5 * (T1 - T0) * erfc((x[mid, 0] - xm) / (2.0 * np.sqrt(kappa * alpha * t)))
    assert np.abs(d.get_field("T")[mid] - exact).max() < 0.015 * (T1 - T0)


def test_jc_yield_table_and_newton_residual():
    """KATs: JC sigma_y from the formula; Newton converges to 1e-10 relative."""
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    d = _oracle(sc, {"return_map": 1})
    d.step(300)
    ps = d.get_field("pl_strain")
    sy = d.get_field("sigma_y")
    eff = d.get_field("eff_strain_rate")
    m = sc["mat"]
    plastic = d.get_field("dep") > 0
    assert plastic.sum() > 10
    # on the yield surface: sigma_y == JC(eps_p, rate, T = 20 C)
    expect = (m.A + m.B * ps ** m.n) * (1 + m.C * np.log(np.where(eff == 0, 1e-5, eff) / m.eps0))
    np.testing.assert_allclose(sy[plastic], expect[plastic], rtol=1e-12)
    # the stress sits on the surface: sigma_eq == sigma_y for plastic particles
    np.testing.assert_allclose(d.get_field("sigma_eq")[plastic], sy[plastic], rtol=1e-12)
    iters = d.get_scalar("newton_iters") / max(1.0, d.get_scalar("newton_calls"))
    assert 0 < iters < 20


def test_radial_equals_newton_for_perfect_plasticity():
    """KAT: with zero hardening the one-step radial return is the Newton solution."""
    sc = S.compression_cylinder()
    sc["mat"].Et = 0.0
    a = _oracle(sc, {"return_map": 0})
    b = _oracle(sc, {"return_map": 1})
    a.step(700)
    b.step(700)
    pa, pb = a.get_field("pl_strain"), b.get_field("pl_strain")
    assert pa.max() > 1e-3
    np.testing.assert_allclose(pb, pa, rtol=1e-9, atol=1e-15)


def test_quirky_tensor_product_by_hand():
    """KAT: tensor3 operator* (src/cuda/tensor3.cu:241-256) on a hand case,
    observed through one stress update with a pure rotation rate."""
    # shear stress S = [[1,2,0],[2,3,0],[0,0,0]] MPa, W with only xy = w
    n = 1
    d = O.OracleDomain(n)
    d.set_h(1.0)
    d.set_density(1.0)
    d.set_shear_modulus(0.0)
    d.set_sigma_y(1e30)
    d.set_time_step(1.0)
    d.set_material(_abi.WfMaterial(model=0, E=1.0, nu=0.3))
    S0 = np.array([[1.0, 3.0, 0.0, 2.0, 0.0, 0.0]])          # flat xx yy zz xy yz xz
    W0 = np.array([[0.0, 0.0, 0.0, 0.5, 0.0, 0.0]])
    d.set_field("shearstress", S0)
    d.set_field("rotrate", W0)
    d.set_field("strrate", np.zeros((1, 6)))
    d.run_stage("stress")
    S = d.get_field("shearstress")[0]
    Sm = np.array([[1.0, 2.0, 0.0], [2.0, 3.0, 0.0], [0.0, 0.0, 0.0]])
    Wm = np.array([[0.0, 0.5, 0.0], [-0.5, 0.0, 0.0], [0.0, 0.0, 0.0]])

    def mul_ref(A, B):       # column x = A.B, columns y,z = A.B^T
        R = np.empty((3, 3))
        R[:, 0] = (A @ B)[:, 0]
        R[:, 1:] = (A @ B.T)[:, 1:]
        return R
    expect = Sm + mul_ref(Sm, Wm.T) + mul_ref(Wm, Sm)
    np.testing.assert_allclose(S, [expect[0, 0], expect[1, 1], expect[2, 2], expect[0, 1],
                                   expect[1, 2], expect[0, 2]], rtol=0, atol=1e-15)


def test_mlp_gradient_check_fp64():
    """Finite differences against the FP64 backward pass of the oracle MLP."""
    rng = np.random.default_rng(3)
    npar = 64 * 4 + 64 + 64 * 64 + 64 + 64 + 1
    P = rng.normal(0, 0.3, npar)
    X = rng.uniform(-1, 1, (16, 4))
    T = rng.uniform(0, 1, 16)
    loss, g = O.mlp_loss_grad(P, X, T)
    for k in rng.choice(npar, 40, replace=False):
        e = np.zeros(npar)
        e[k] = 1e-6
        lp, _ = O.mlp_loss_grad(P + e, X, T)
        lm, _ = O.mlp_loss_grad(P - e, X, T)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), k


@pytest.mark.skipif(O.ref_lib() is None and build_ref.build() is None,
                    reason="reference tree not present (golden vectors cover this machine)")
def test_oracle_matches_reference_live_cylinder_r5mm_neighbors_and_steps():
    """The R 5 mm, H 10 mm cylinder (5,244 particles): neighbour lists and 50 Fraser steps,
    reference kernels vs oracle, bit for bit."""
    O._ref = None
    c1 = S.compression_cylinder(R=0.005, H=0.010)
    cr, lr = O.ref_neighbors(c1["x"], c1["h"])
    d = _oracle(c1)
    d.find_neighbors()
    co, lo = d.get_neighbors()
    assert np.array_equal(cr, co)
    assert all(np.array_equal(lr[i, :cr[i]], lo[i, :co[i]]) for i in range(len(cr)))
    R = S.load_ref(O.RefDomain(c1["n"]), c1)
    R.begin()
    R.step(50)
    d2 = _oracle(c1)
    d2.step(50)
    for f in ("x", "v", "sigma", "rho", "int_energy"):
        assert np.array_equal(R.get(f), d2.get_field(f)), f


def test_oracle_output_rows_are_the_reductions_of_its_fields():
    """The oracle's output rows (every step) are the plain reductions of its
    own fields: maxima of u and pl_strain from 0, the energy sum, and each BC
    zone's load m a before the BC; the platen load of a compression run is
    compressive on the body (the top zone is pushed up: +z on the body's zone
    particles) and grows with the plastic strain."""
    sc = S.compression_cylinder(R=0.003, H=0.006)
    d = _oracle(sc, {"output_every_step": 1})
    d.step(60)
    rows = d.get_output_series()
    assert rows.shape == (60, 11 + 6)
    assert np.array_equal(rows[:, 1], np.arange(1, 61))
    u, ps, e = d.get_field("u"), d.get_field("pl_strain"), d.get_field("int_energy")
    last = rows[-1]
    assert last[2] == max(0.0, u[:, 0].max()) and last[4] == max(0.0, u[:, 2].max())
    assert last[5] == max(0.0, ps.max())
    assert abs(last[10] - e.sum()) <= 1e-12 * np.abs(e).sum()
    assert np.all(rows[:, 6:10] == 0.0)                 # no contact
    fz_top = rows[:, 11 + 3 + 2]
    assert fz_top[-1] > 0.0 and fz_top[-1] > fz_top[5]


def test_oracle_newton_cap_counted():
    sc = S.compression_cylinder(R=0.003, H=0.006, material="jc", vz_top=-10.0)
    d = _oracle(sc, {"return_map": 1, "newton_max_iter": 1})
    d.step(200)
    assert d.get_scalar("newton_calls") > 0
    assert d.get_scalar("newton_capped") == d.get_scalar("newton_calls")
    ok = _oracle(sc, {"return_map": 1})
    ok.step(200)
    assert ok.get_scalar("newton_capped") == 0


@pytest.mark.parametrize("k", [1, 100, 500])
def test_heat_oracle_matches_reference_thermal_golden(k):
    """Heat only (ThermalSolve): the oracle's conduction, convection and
    leapfrog on the 16^3 heat box against the reference's own Thermal.cu
    kernels (golden vectors), bit for bit at steps 1, 100 and 500."""
    g = np.load(os.path.join(GOLDEN, "thermal_box.npz"))
    hb = S.heat_box(n_side=16)
    o = S.load_heat(O.OracleDomain(hb["n"]), hb)
    o.thermal_solve((k - 0.5) * hb["dt"])
    assert o.get_scalar("step") == k
    for f in ("T", "Ta", "Tb", "dTdt"):
        assert np.array_equal(o.get_field(f), g["s%d_%s" % (k, f)]), f


def test_heat_oracle_matches_reference_thermal_live():
    """The same against the reference's Thermal.cu kernels run here (skipped
    where the reference tree is absent)."""
    O._ref = None
    if build_ref.build() is None or O.ref_lib() is None:
        pytest.skip("reference tree not present")
    hb = S.heat_box(n_side=12)
    R = O.RefDomain(hb["n"])
    R.thermal_solve(hb, 200)
    o = S.load_heat(O.OracleDomain(hb["n"]), hb)
    o.thermal_solve(199.5 * hb["dt"])
    for f in ("T", "Ta", "Tb", "dTdt"):
        assert np.array_equal(o.get_field(f), R.get(f)), f
