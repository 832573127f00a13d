"""The learned warm start: training kernels checked against the FP64 oracle,
tensor-core inference against FP32/FP64, the gain over the radial start, and
its use inside the solver (which must not change the converged answer)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import scenarios as S

pytestmark = pytest.mark.gpu


def jc_mat():
    sc = S.compression_cylinder(material="jc")
    return sc["mat"], sc["G"]


def test_training_gradient_matches_fp64_oracle():
    from weldformgpu_gb300 import mlp
    rng = np.random.default_rng(5)
    P = mlp.init_params(3)
    X = rng.uniform(-1, 1, (1000, 4)).astype(np.float32)
    Y = rng.uniform(0, 1, 1000).astype(np.float32)
    loss, g = mlp.grad(P, X, Y)
    lo, go = O.mlp_loss_grad(P.astype(np.float64), X.astype(np.float64), Y.astype(np.float64))
    assert abs(loss - lo) <= 1e-5 * abs(lo)
    # FP32 accumulation over 1000 samples: relative L2 error of the whole gradient
    err = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert err < 1e-4, err


def test_tensor_core_inference_close_to_fp64():
    from weldformgpu_gb300 import mlp
    rng = np.random.default_rng(6)
    P = mlp.init_params(4)
    X = rng.uniform(-1, 1, (5000, 4)).astype(np.float32)
    y64 = O.mlp_forward(P.astype(np.float64), X.astype(np.float64))
    y32 = mlp.infer(P, X, tensor_cores=False)
    ytc = mlp.infer(P, X, tensor_cores=True)
    np.testing.assert_allclose(y32, y64, rtol=1e-5, atol=1e-5)
    # BF16 operands (8-bit mantissa), FP32 accumulation
    assert np.max(np.abs(ytc - y64)) < 0.05 * np.max(np.abs(y64)) + 0.02
    assert np.corrcoef(ytc, y64)[0, 1] > 0.999


def _bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def test_tensor_core_inference_matches_bf16_forward():
    """The tcgen05 path against a CPU forward that rounds like it: layer 1 in
    FP32, its SiLU (h + h tanh h, h = z/2) rounded to BF16, W2 in BF16, layer 2
    accumulated exactly, layer 3 in FP64.  Per sample the difference is
    bounded by what the GPU rounds differently: its tanh.approx.bf16x2 in
    layer 1 may land one BF16 step (2^-8 relative) away, and its
    tanh.approx.f32 in layer 3 carries a relative error below 2^-10 -- so
    |dy| <= sum_j |w3_j| (2^-10 |s_j| + 1.1 * 2^-7 sum_k |W2_jk| |a_k|) + 1e-6,
    about a hundred times tighter than the FP64 comparison above."""
    from weldformgpu_gb300 import mlp
    rng = np.random.default_rng(7)
    P = mlp.init_params(5).astype(np.float32)
    P[256:320] = rng.normal(0.0, 0.2, 64)        # non-zero biases b1, b2
    P[4416:4480] = rng.normal(0.0, 0.2, 64)
    X = rng.uniform(-1, 1, (4096, 4)).astype(np.float32)
    W1 = P[:256].reshape(64, 4).astype(np.float64)
    b1 = P[256:320].astype(np.float64)
    W2 = _bf16(P[320:4416]).reshape(64, 64).astype(np.float64)
    b2 = P[4416:4480].astype(np.float64)
    W3 = P[4480:4544].astype(np.float64)
    b3 = float(P[4544])
    z1 = (X.astype(np.float64) @ W1.T + b1).astype(np.float32)
    h = _bf16(0.5 * z1).astype(np.float64)
    t = _bf16(np.tanh(h).astype(np.float32)).astype(np.float64)
    a = _bf16((h * t + h).astype(np.float32)).astype(np.float64)
    v = a @ W2.T + b2
    sv = 0.5 * v
    y_emu = (W3 * (sv * np.tanh(sv) + sv)).sum(axis=1) + b3
    bound = (np.abs(W3) * (2.0 ** -10 * np.abs(sv) +
                           1.1 * 2.0 ** -7 * (np.abs(a) @ np.abs(W2).T))).sum(axis=1) + 1e-6
    ytc = mlp.infer(P, X, tensor_cores=True).astype(np.float64)
    err = np.abs(ytc - y_emu)
    assert np.all(err <= bound), (err.max(), bound[np.argmax(err / bound)], (err / bound).max())
    assert np.median(err) < 0.1 * np.median(bound)


def _gain(mat, G, steps):
    from weldformgpu_gb300 import mlp
    P, loss = mlp.train_jc_warm_start(mat, G, n_synth=131072, steps=steps)
    _, Yt, St, it_synth = mlp.synth(mat, G, 20000, seed=11, rtol=1e-10)
    it_r, used_r, dl_r = mlp.newton_iters(mat, G, None, St, rtol=1e-10)
    it_m, used_m, dl_m = mlp.newton_iters(mat, G, P, St, rtol=1e-10)
    # same solver and tolerance (states re-read from their FP32 copies)
    assert abs(it_r.mean() - it_synth.mean()) < 0.05
    assert not used_r.any() and used_m.mean() > 0.95
    # the start changes the iteration count only: same converged increment
    np.testing.assert_allclose(dl_m, dl_r, rtol=1e-6)
    return loss, it_r.mean(), it_m.mean()


def test_network_gain_on_the_benchmark_material():
    """Al Johnson-Cook (B = 114 MPa, n = 0.42): hardening is weak against 3G,
    the radial start is within ~10% of the converged increment and Newton
    needs 1-2 iterations.  The network may not make it worse."""
    mat, G = jc_mat()
    loss, it_r, it_m = _gain(mat, G, 2500)
    print("Al JC: MSE %.2e, Newton iterations radial %.3f, MLP %.3f" % (loss, it_r, it_m))
    assert loss < 1e-3
    assert it_m <= it_r + 0.05


def test_network_gain_on_stiff_hardening():
    """Stiff hardening (B = 20 GPa, n = 0.3): the radial start overshoots by up
    to 50x and Newton needs ~4 iterations; the trained start cuts that."""
    mat, G = jc_mat()
    mat.B, mat.n = 20e9, 0.3
    loss, it_r, it_m = _gain(mat, G, 4000)
    print("stiff JC: MSE %.2e, Newton iterations radial %.3f, MLP %.3f" % (loss, it_r, it_m))
    assert it_r > 3.0
    assert it_m < 0.75 * it_r, (it_m, it_r)


def test_plain_solver_logs_training_pairs():
    from weldformgpu_gb300 import Domain_d
    sc = S.compression_cylinder(material="jc", vz_top=-10.0)
    d = S.load(Domain_d(sc["n"]), sc, {"return_map": 1, "log_return_map": 20000})
    d.step(300)
    X, Y = d.get_return_map_log(20000)
    assert len(X) > 1000
    assert np.all(Y > 0) and np.all(Y <= 1.0 + 1e-6)
    assert np.all(X[:, 0] >= 0)                  # trial ratio - 1


def test_mlp_in_solver_same_answer():
    from weldformgpu_gb300 import Domain_d, mlp
    mat, G = jc_mat()
    P, _ = mlp.train_jc_warm_start(mat, G, n_synth=65536, steps=1500)
    sc = S.compression_cylinder(R=0.004, H=0.008, material="jc", vz_top=-10.0,
                                generator="lattice", dt_rule="sound_speed")
    opts = {"return_map": 1, "precision": 1}
    a = S.load(Domain_d(sc["n"]), sc, opts)
    b = S.load(Domain_d(sc["n"]), sc, opts)
    b.set_mlp_weights(P)
    b.set_option("mlp", 1)
    a.step(500)
    b.step(500)
    assert a.get_field("pl_strain").max() > 0.005
    assert b.get_scalar("mlp_used") > 0
    # both starts converge to the same residual tolerance
    for f in ("pl_strain", "sigma_eq", "u"):
        ref = a.get_field(f)
        np.testing.assert_allclose(b.get_field(f), ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())
