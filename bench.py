"""Benchmark of the explicit SPH step: particle-steps/s on one GB300.

Workload: coupled thermo-mechanical Johnson-Cook
cylinder compression, R = 25 mm, H = 50 mm, dx = 0.5 mm, seeded jittered
lattice (~0.79M particles), consistent Newton return map, Taylor-Quinney
plastic heat, platen at -10 m/s.  A "step" is one pass of the Fraser loop
body over all particles (density, rates + stress, acceleration, integration,
heat, neighbour rebuild every 5 steps).

`value` is the mixed-precision form (FP32 pair loops / stress / flux, FP64
positions, velocities, plastic strain, Newton, reductions; MLP warm start
when trained weights are loaded) with inputs resident in HBM; `plain_fp64`
is the plain-FP64 form of the same code; `e2e` times the drop-in call
(create, setters from host arrays, solve, read-back of the output fields)
with host clocks.  `cpu_baseline` times the FP64 CPU oracle on the host cores.
`rel_l2_vs_fp64` compares the two forms from the same plastic state after the
timed steps; `rel_l2_vs_fp64_from_rest` over a 5,000-step run from rest of a
smaller cylinder of the same material and loading; `fp64_ceiling` puts the
plain form against the measured FP64 FMA throughput; `heat` and `indentation`
are the 1M-particle heat-only and 2M-particle contact workloads.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s, mixed+MLP vs plain FP64 on 1 GB300 at ≤1e-3 rel L2 err"
UNIT = "particle-steps/s"
WORKLOAD = "jc_thermomech_compression_R25mm_H50mm_dx0.5mm"

# Algorithmic bytes per particle for each kernel: every per-particle field the
# kernel reads or writes, once, in the form it is stored (neighbour gathers are
# served by L1/L2; the neighbour-index list is counted separately).  In the
# mixed form the density launch also runs the previous step's heat pass
# (k_density_heat32); "thermal" there is only the heat pass of a call's last step.
BYTES_MODEL = {
    "mixed": {"density": 216, "stress": 248, "accel": 96, "integrate": 320, "thermal": 88},
    "fp64": {"density": 120, "stress": 416, "accel": 144, "integrate": 264, "thermal": 112},
}
# Bytes of one launch of the mixed form's kernels as timed (no contact): the
# density launch carries the previous step's heat pass (216 + 88) and the
# acceleration launch the integration of the same slot (96 + 320).
LAUNCH_BYTES_MIXED = {"density": 216 + 88, "stress": 248, "accel": 96 + 320, "thermal": 88}
NB_INDEX_BYTES = 4  # per neighbour per pair pass
KERNEL_IDS = {"density": 1, "stress": 2, "accel": 3, "integrate": 4, "thermal": 5}
TOP_FZ = 11 + 3 * 1 + 2     # output-row column: BC 1 (the moving platen zone), z component
PAIR_KERNELS = ("density", "stress", "accel", "thermal")


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


class ProfilerRange:
    """cuProfilerStart/Stop around a timed region, so that `ncu
    --profile-from-start off` captures only the timed steps; without a
    profiler attached both calls do nothing."""

    def __enter__(self):
        self.lib = None
        try:
            import ctypes
            self.lib = ctypes.CDLL("libcuda.so.1")
            self.lib.cuProfilerStart()
        except OSError:
            self.lib = None
        return self

    def __exit__(self, *a):
        if self.lib is not None:
            self.lib.cuProfilerStop()


def build_domain(sc, opts):
    from weldformgpu_gb300 import Domain_d
    from weldformgpu_gb300 import scenarios as S
    return S.load(Domain_d(sc["n"]), sc, opts)


def base_options():
    return {"return_map": 1, "thermal": 1, "taylor_quinney": 0.9, "rebuild_every": 5,
            "rebuild_current_positions": 1, "rebuild_after_yield": 0, "energy_mode": 1}


def per_kernel_ms(d, kernels, reps=1):
    """Event-timed duration of each kernel kind over `reps` steps each."""
    out = {}
    for k in kernels:
        d.set_option("profile_kernel", KERNEL_IDS[k])
        _, kms, kl, _ = d.time_steps(reps)
        out[k] = kms / max(kl, 1)
    d.set_option("profile_kernel", 0)
    return out


def preload(sc, steps):
    """Runs the mixed form from rest for `steps` steps and returns a checkpoint
    (host arrays): the timed runs start from this plastic state."""
    opts = base_options()
    opts["precision"] = 1
    d = build_domain(sc, opts)
    d.step(steps)
    st = d.checkpoint()
    st["_plastic_fraction"] = float(np.mean(st["pl_strain"] > 0))
    d.close()
    return st


MLP_SYNTH = 1 << 21          # synthetic states (targets from an FP64 Newton on the GPU)
MLP_STEPS = 8000             # Adam steps of 4,096 pairs (~3 passes over ~10.5M pairs)


def train_mlp(sc, state, log_steps=12, cap=1 << 23):
    """Warm-start network for this material: ~10M training pairs, the
    (state, converged increment) pairs the plain FP64 form logs over
    `log_steps` steps from the checkpoint (up to `cap`, ~0.7M plastic
    particles per step at 786k) plus MLP_SYNTH synthetic states, trained on
    the GPU."""
    from weldformgpu_gb300 import mlp
    t0 = time.perf_counter()
    opts = base_options()
    opts["precision"] = 0
    d = build_domain(sc, opts)
    d.restore(state)
    d.set_option("log_return_map", cap)
    d.step(log_steps)
    logged = d.get_return_map_log(cap)
    d.close()
    params, loss = mlp.train_jc_warm_start(sc["mat"], sc["G"], n_synth=MLP_SYNTH, logged=logged,
                                           steps=MLP_STEPS, batch=4096)
    info = {"train_loss_mse": loss, "logged_pairs": int(len(logged[0])),
            "synthetic_pairs": MLP_SYNTH, "train_steps": MLP_STEPS, "batch": 4096,
            "train_s": time.perf_counter() - t0}
    return params, info


def run_form(sc, form, steps, warmup, state, mlp_params=None, extra_opts=None):
    opts = base_options()
    opts["precision"] = 1 if form == "mixed" else 0
    opts.update(extra_opts or {})
    d = build_domain(sc, opts)
    d.restore(state)
    if mlp_params is not None:
        d.set_mlp_weights(mlp_params)
        d.set_option("mlp", 1)
    d.step(warmup)
    kernels = ["density", "stress", "accel", "integrate", "thermal"]
    kms = per_kernel_ms(d, kernels, reps=20)
    dominant = max(kms, key=kms.get)
    d.set_option("profile_kernel", KERNEL_IDS[dominant])
    it0, c0 = d.get_scalar("newton_iters"), d.get_scalar("newton_calls")
    u0 = d.get_scalar("mlp_used")
    with ClockSampler() as clk, ProfilerRange():
        elapsed, kernel_ms, kernel_launches, launches = d.time_steps(steps)
    d.set_option("profile_kernel", 0)
    it1, c1 = d.get_scalar("newton_iters"), d.get_scalar("newton_calls")
    u1 = d.get_scalar("mlp_used")
    # 20 more steps with an output row every step: the reaction curve of both forms
    d.set_option("output_every_step", 1)
    d.step(20)
    rows = d.get_output_series()[-20:]
    fields = {f: d.get_field(f) for f in ("u", "pl_strain", "sigma_eq", "T")}
    fields["reaction_force"] = rows[:, TOP_FZ]
    d.close()
    return dict(elapsed_ms=elapsed, kernel_ms=kernel_ms, kernel_launches=kernel_launches,
                launches=launches, dominant=dominant, per_kernel_ms=kms, clocks=clk.summary(),
                newton_iters_per_call=(it1 - it0) / max(c1 - c0, 1.0),
                plastic_per_step=(c1 - c0) / max(steps, 1),
                mlp_used_per_step=(u1 - u0) / max(steps, 1), fields=fields)


_PINNED = []   # the tensors that own the pinned pages of pinned_like arrays


def pinned_like(a):
    """A copy of host array `a` in page-locked (pinned) host memory."""
    import torch
    t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
    _PINNED.append(t)
    out = t.numpy()
    out[...] = a
    return out


def e2e_call(sc, form, steps, state, mlp_params=None, outs=None):
    """One drop-in call from host buffers, host wall clock around everything:
    create, setters, restore from the checkpoint, solve, read-back, destroy."""
    from weldformgpu_gb300 import Domain_d
    from weldformgpu_gb300 import scenarios as S
    opts = base_options()
    opts["precision"] = 1 if form == "mixed" else 0
    n = sc["n"]
    fields = ("u", "pl_strain", "sigma_eq", "T")
    t0 = time.perf_counter()
    d = S.load(Domain_d(n), sc, opts)
    d.restore(state)
    if mlp_params is not None:
        d.set_mlp_weights(mlp_params)
        d.set_option("mlp", 1)
    d.step(steps)
    out = [d.get_field(f, out=None if outs is None else outs[f]) for f in fields]
    d.close()
    t1 = time.perf_counter()
    h2d = n * (3 * 8 + 8 + 4 + 1 + 8)               # scenario: x, m, id, not_write, T (Cs stays on the host)
    h2d += sum(v.nbytes for k, v in state.items() if not k.startswith("_"))
    d2h = sum(a.nbytes for a in out)
    return n * steps / (t1 - t0), h2d / steps, d2h / steps


def run_e2e(sc, form, steps, state, mlp_params=None, reps=3):
    """The end-to-end arm: inputs (scenario arrays and the checkpoint) and the
    output buffers in pinned host memory, allocated before the timed calls;
    one untimed warm-up call, then the median of `reps` timed calls (each a
    complete create ... destroy)."""
    psc = {k: (pinned_like(v) if isinstance(v, np.ndarray) else v) for k, v in sc.items()}
    psc["Cs_particles"] = pinned_like(np.full(sc["n"], sc["Cs"]))
    pstate = {k: (pinned_like(v) if isinstance(v, np.ndarray) else v) for k, v in state.items()}
    n = sc["n"]
    outs = {"u": pinned_like(np.zeros(3 * n)), "pl_strain": pinned_like(np.zeros(n)),
            "sigma_eq": pinned_like(np.zeros(n)), "T": pinned_like(np.zeros(n))}
    e2e_call(psc, form, steps, pstate, mlp_params, outs)
    runs = [e2e_call(psc, form, steps, pstate, mlp_params, outs) for _ in range(reps)]
    vals = sorted(r[0] for r in runs)
    return vals[len(vals) // 2], runs[0][1], runs[0][2]


def cpu_baseline(sc, budget_s=12.0):
    """FP64 CPU oracle (all host threads) on the same workload, bounded sample."""
    from oracle import oracle as O
    from weldformgpu_gb300 import scenarios as S
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    opts = base_options()
    d = S.load(O.OracleDomain(sc["n"]), sc, opts)
    d.step(1)                                      # set-up + neighbour search + 1 step
    t0 = time.perf_counter()
    done = 0
    while True:
        d.step(1)
        done += 1
        if time.perf_counter() - t0 > budget_s or done >= 50:
            break
    dt = time.perf_counter() - t0
    return {"value": sc["n"] * done / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d Fraser steps (after 1 set-up step) of the full %d-particle workload, "
                      "FP64 oracle (oracle/wf_oracle.c), OpenMP" % (done, sc["n"])}


def rel_l2(a, b):
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


FROM_REST = {"R": 0.010, "H": 0.020, "steps": 5000}
FROM_REST_FIELDS = ("u", "pl_strain", "sigma_eq", "T", "reaction_force")


def from_rest_errors(mlp_params=None, steps=None):
    """Both forms from rest on a smaller cylinder of the same material, dx,
    loading and options (R = 10 mm, H = 20 mm, ~50k particles) for `steps`
    steps (default 5,000: 12 % height reduction; 20,000: 49 %): relative L2
    error of the mixed form (with the network when given) against the plain
    FP64 form on the output fields and on the platen's reaction curve (an
    output row every step), at the end and, for longer runs, every 5,000
    steps."""
    from weldformgpu_gb300 import scenarios as S
    steps = steps or FROM_REST["steps"]
    sc = S.jc_compression(R=FROM_REST["R"], H=FROM_REST["H"])
    doms, secs = {}, {"fp64": 0.0, "mixed": 0.0}
    for form in ("fp64", "mixed"):
        opts = base_options()
        opts["precision"] = 1 if form == "mixed" else 0
        opts["output_every_step"] = 1
        opts["output_series_cap"] = steps + 16
        d = build_domain(sc, opts)
        if form == "mixed" and mlp_params is not None:
            d.set_mlp_weights(mlp_params)
            d.set_option("mlp", 1)
        doms[form] = d
    checkpoints, done, max_ps = [], 0, 0.0
    while done < steps:
        k = min(5000, steps - done)
        for form, d in doms.items():
            t0 = time.perf_counter()
            d.step(k)
            secs[form] += time.perf_counter() - t0
        done += k
        out = {}
        for form, d in doms.items():
            out[form] = {f: d.get_field(f) for f in ("u", "pl_strain", "sigma_eq", "T")}
            out[form]["reaction_force"] = d.get_output_series()[:, TOP_FZ]
        errs = {f: rel_l2(out["mixed"][f] - (20.0 if f == "T" else 0.0),
                          out["fp64"][f] - (20.0 if f == "T" else 0.0)) for f in FROM_REST_FIELDS}
        max_ps = float(out["fp64"]["pl_strain"].max())
        errs.update({"steps": done, "max_pl_strain": max_ps,
                     "height_reduction": float(-out["fp64"]["u"].reshape(-1, 3)[:, 2].min()
                                               / FROM_REST["H"])})
        checkpoints.append(errs)
    for d in doms.values():
        d.close()
    errs = {f: checkpoints[-1][f] for f in FROM_REST_FIELDS}
    errs.update({"steps": steps, "particles": sc["n"],
                 "workload": "jc_thermomech_compression_R10mm_H20mm_dx0.5mm from rest",
                 "max_pl_strain": max_ps, "height_reduction": checkpoints[-1]["height_reduction"],
                 "fp64_run_s": secs["fp64"], "mixed_run_s": secs["mixed"],
                 "mlp": mlp_params is not None})
    if len(checkpoints) > 1:
        errs["checkpoints"] = checkpoints
    return errs


def fp64_ceiling(plain_per_kernel_ms, n):
    """The plain form against the measured FP64 FMA throughput: FP64 flops per
    particle of each pair kernel (ncu instruction counts, profiles/fp64_flops.json:
    2 per DFMA, 1 per DADD / DMUL) over its event-timed duration."""
    import ctypes as C
    from weldformgpu_gb300 import domain as D
    g, ms = C.c_double(), C.c_double()
    rc = D.lib().wf_fp64_fma_peak(C.byref(g), C.byref(ms))
    if rc != 0:
        return None
    out = {"peak_gflops": g.value, "peak_kind": "measured (wf_fp64_fma_peak: FMA chains on every SM)"}
    fp = os.path.join(ROOT, "profiles", "fp64_flops.json")
    if os.path.exists(fp):
        with open(fp) as f:
            flops = json.load(f)["fp64"]
        per = {}
        for k, fpp in flops.items():
            if k in plain_per_kernel_ms and plain_per_kernel_ms[k] > 0:
                a = fpp * n / (plain_per_kernel_ms[k] / 1e3) / 1e9
                per[k] = {"flops_per_particle": fpp, "achieved_gflops": a,
                          "frac": a / g.value}
        out["kernels"] = per
        tot = sum(flops.values())
        out["flops_per_particle_step"] = tot
    return out


def dist_setup(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist.init_process_group("gloo")
    return rank, ws, dist


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def indentation_domain(sc, form, shift_t, state=None):
    """The indentation workload's domain: the tool's nodes moved by its velocity
    times `shift_t` (the tool translates at constant velocity, so this is where
    a run of that length leaves it), particle state restored from `state`."""
    sc2 = dict(sc)
    ms = dict(sc["mesh"])
    ms["nodes"] = ms["nodes"] + np.asarray(ms["vel"]) * shift_t
    sc2["mesh"] = ms
    opts = base_options()
    opts["precision"] = 1 if form == "mixed" else 0
    d = build_domain(sc2, opts)
    if state is not None:
        d.restore(state)
    return d


def bench_indentation(args):
    """Indentation workload (--size full): block 200 x 200 x 50 at dx = 0.25 mm (2.0M particles;
    medium 100 x 100 x 50, small 50 x 50 x 25)
    indented by the lower half of a level-5 icosphere (R = 10 mm, 10,304
    triangles) at -5 m/s; contact law 1 (0.1 K/dx penalty, mu = 0.3,
    frictional heat), JC, coupled heat, neighbour rebuild at a plastic-strain
    increment of 0.05.  The mixed form runs `--preload` steps from rest to
    develop the contact; both forms are timed from that state."""
    from weldformgpu_gb300 import scenarios as S
    L = {"full": (0.05, 0.05, 0.0125), "medium": (0.025, 0.025, 0.0125),
         "small": (0.0125, 0.0125, 0.00625)}[args.size]
    sc = S.indent_block(L=L, dx=0.00025, R=0.01, level=5, v_tool=-5.0, mu=0.3, thermal=True,
                        rebuild_increment=0.05)
    ns, ne = sc["n_solid"], len(sc["mesh"]["tris"])
    preload = args.preload if args.preload != 4000 else 1000
    d = indentation_domain(sc, "mixed", 0.0)
    d.step(preload)
    state = d.checkpoint()
    t_pre = state["_time"]
    contacts_pre = int((d.get_field_i32("cont_count") > 0).sum())
    d.close()
    forms = [f for f in ("mixed", "fp64") if f in args.forms.split(",")]
    out = {}
    for form in forms:
        steps = args.steps if form == "mixed" else max(3, args.steps // 20)
        d = indentation_domain(sc, form, t_pre, state)
        d.step(max(args.warmup, 3))
        kms = per_kernel_ms(d, ["density", "stress", "accel", "integrate", "thermal"], reps=5)
        d.set_option("profile_kernel", 7)
        _, cms, cl, _ = d.time_steps(5)
        kms["contact"] = cms / max(cl / 2, 1)          # two timed scopes per step
        d.set_option("profile_kernel", 0)
        r0 = d.get_scalar("rebuilds")
        with ClockSampler() as clk, ProfilerRange():
            elapsed, _, _, launches = d.time_steps(steps)
        out[form] = dict(value=ns * steps / (elapsed / 1e3), ms_per_step=elapsed / steps,
                         per_kernel_ms=kms, launches=launches, clocks=clk.summary(),
                         rebuilds_per_step=(d.get_scalar("rebuilds") - r0) / steps,
                         contacts=int((d.get_field_i32("cont_count") > 0).sum()))
        d.close()
    line = {"workload": "indentation_block%dx%dx%d_dx0.25mm_icosphere_R10mm_level5" % tuple(
                int(round(v / 0.00025)) for v in L),
            "metric": "particle-steps/s (solid particles), mixed vs plain FP64 on 1 GB300",
            "unit": UNIT, "value": out["mixed"]["value"], "ms_per_step": out["mixed"]["ms_per_step"],
            "steps": args.steps, "n_gpus": 1, "dtype": "f32+f64", "data": "synthetic",
            "config": {"solid_particles": ns, "rigid_particles": ne, "triangles": ne,
                       "dx_m": sc["dx"], "dt_s": sc["dt"], "tool_velocity_m_s": -5.0,
                       "contact": "law 1: 0.1 K/dx penalty, mu 0.3, frictional heat",
                       "rebuild": "plastic-strain increment 0.05", "preload_steps": preload,
                       "contacts_at_start": contacts_pre},
            "mixed": out["mixed"]}
    if "fp64" in out:
        # parity of the two forms over 20 steps from the same state
        fields = {}
        for form in ("mixed", "fp64"):
            d = indentation_domain(sc, form, t_pre, state)
            d.step(20)
            fields[form] = {f: d.get_field(f) for f in ("u", "pl_strain", "sigma_eq", "T",
                                                        "contforce")}
            d.close()
        line["plain_fp64"] = out["fp64"]
        line["speedup_vs_plain_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
        line["rel_l2_vs_fp64_after_20_steps"] = {
            f: rel_l2(fields["mixed"][f] - (20.0 if f == "T" else 0.0),
                      fields["fp64"][f] - (20.0 if f == "T" else 0.0)) for f in fields["mixed"]}
    return line


def bench_heat(args):
    """Heat-only workload: heat conduction only (ThermalSolve) in a 100^3-particle
    steel box (dx = 0.1 mm, 1.0M particles), Gaussian hot spot, convection on
    the outer layer, dt = 0.1 dx^2 rho c_p / k.  Plain FP64 against the mixed
    form (FP32 flux, FP64 temperature accumulation).  Each solve call starts
    with one neighbour search (as the reference's ThermalSolve) and is timed
    with the host clock around the call after one warm-up call."""
    from weldformgpu_gb300 import Domain_d
    from weldformgpu_gb300 import scenarios as S
    sc = S.heat_box(n_side=100)
    n = sc["n"]
    steps = max(args.steps, 20) * 2
    out, T = {}, {}
    for form in ("mixed", "fp64"):
        d = S.load_heat(Domain_d(n), sc)
        d.set_option("precision", 1 if form == "mixed" else 0)
        d.thermal_solve(5 * sc["dt"])
        t0 = time.perf_counter()
        d.thermal_solve(steps * sc["dt"] * (1.0 - 1e-9))
        el = time.perf_counter() - t0
        T[form] = d.get_field("T")
        out[form] = dict(value=n * steps / el, ms_per_step=1e3 * el / steps,
                         steps=int(d.get_scalar("step")) - 5)
        d.close()
    line = {"workload": "heat_conduction_box100x100x100_dx0.1mm", "unit": UNIT,
            "metric": "particle-steps/s, mixed (FP32 flux) vs plain FP64 on 1 GB300",
            "value": out["mixed"]["value"], "ms_per_step": out["mixed"]["ms_per_step"],
            "steps": steps, "n_gpus": 1, "dtype": "f32+f64", "data": "synthetic",
            "config": {"particles": n, "dx_m": sc["dx"], "dt_s": sc["dt"],
                       "timing": "host clock around one ThermalSolve call of `steps` steps, "
                                 "including its initial neighbour search"},
            "mixed": out["mixed"], "plain_fp64": out["fp64"],
            "speedup_vs_plain_fp64": out["mixed"]["value"] / out["fp64"]["value"],
            "rel_l2_vs_fp64": rel_l2(T["mixed"] - sc["T"], T["fp64"] - sc["T"])}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="small workload (quick check)")
    ap.add_argument("--size", default="full", choices=["full", "medium", "small"],
                    help="full: R=25 mm H=50 mm (0.79M); medium: R=15 mm H=30 mm (0.17M, > L2); "
                         "small: R=6 mm H=12 mm")
    ap.add_argument("--forms", default="fp64,mixed", help="forms to time (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-oracle baseline")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end arm")
    ap.add_argument("--no-mlp", action="store_true", help="time the mixed form without the MLP")
    ap.add_argument("--from-rest-steps", type=int, default=None,
                    help="length of the from-rest mixed-vs-FP64 comparison (default 5000)")
    ap.add_argument("--tiles", type=int, default=None,
                    help="profiling runs: option tile_staging for the timed form")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the from-rest error run, the FP64 ceiling and the heat / "
                         "indentation workloads")
    ap.add_argument("--preload", type=int, default=4000,
                    help="steps run (mixed form) before the timed runs, to reach plasticity")
    ap.add_argument("--workload", default="compression",
                    choices=["compression", "indentation", "heat"],
                    help="compression: the metric's workload; indentation: the 2M-particle "
                         "contact case; heat: the 1M-particle heat-only case (separate "
                         "lines, not the metric)")
    args = ap.parse_args()
    warmup = max(args.warmup, 3)
    if args.workload in ("indentation", "heat"):
        from weldformgpu_gb300 import build as Bld
        Bld.build()
        print(json.dumps((bench_indentation if args.workload == "indentation" else bench_heat)(args)))
        return
    rank, ws, dist = dist_setup(args.gpus)

    from weldformgpu_gb300 import scenarios as S
    size = "small" if args.small else args.size
    dims = {"full": {}, "medium": {"R": 0.015, "H": 0.030}, "small": {"R": 0.006, "H": 0.012}}[size]
    if args.impl == "reference":
        # the reference arm builds the same workload with the oracle's generator
        # twins: it neither builds nor loads the CUDA library
        from oracle import oracle as O
        sc = S.jc_compression(gen=O, **dims)
    else:
        from weldformgpu_gb300 import build as B
        B.build()
        sc = S.jc_compression(**dims)
    n = sc["n"]
    config = {"workload": WORKLOAD if size == "full" else WORKLOAD + "_" + size, "particles": n,
              "dx_m": sc["dx"], "dt_s": sc["dt"], "nnb": 56, "rebuild_every": 5,
              "return_map": "jc_newton_rtol1e-10", "thermal": "coupled, Taylor-Quinney 0.9",
              "l2": (("inputs larger than L2 (state %.0f MB > 129 MB)" if n * 1100 > 129e6 else
                      "inputs within L2 (state %.0f MB < 129 MB): a reduced case, not a timing run")
                     % (n * 1100 / 1e6)),
              "parallelism": "replicas" if ws > 1 else "single",
              "preload_steps": args.preload}

    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_baseline(sc, budget_s=max(5.0, min(30.0, 1.5 * args.steps)))
        # the CPU arm times steps from the generated state (after one set-up
        # step), not from the preloaded plastic state of the GPU arm
        config = dict(config, preload_steps=0)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
                "n_gpus": args.gpus, "steps": args.steps, "warmup": warmup,
                "higher_is_better": True, "data": "synthetic", "dtype": "f64",
                "config": config, "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "note": "reference CPU path = the FP64 oracle port (the reference's kernels "
                        "compiled for the CPU exist only where the reference tree is present)"}
        print(json.dumps(line))
        return

    state = preload(sc, args.preload)
    forms = args.forms.split(",")
    if "fp64" not in forms or "mixed" not in forms:
        # a profiling run of one form (e.g. under ncu)
        form = "mixed" if "mixed" in forms else "fp64"
        mlp = None if (args.no_mlp or form == "fp64") else train_mlp(sc, state)[0]
        extra = None if args.tiles is None else {"tile_staging": args.tiles}
        r = run_form(sc, form, args.steps, warmup, state, mlp, extra_opts=extra)
        print(json.dumps({"profiling_run": True, "form": form,
                          "ms_per_step": r["elapsed_ms"] / args.steps,
                          "per_kernel_ms": r["per_kernel_ms"], "particles": n}))
        return
    mlp, mlp_info = (None, None) if args.no_mlp else train_mlp(sc, state)
    mixed = run_form(sc, "mixed", args.steps, warmup, state, mlp)
    mixed_nomlp = run_form(sc, "mixed", args.steps, warmup, state) if mlp is not None else None
    plain = run_form(sc, "fp64", args.steps, warmup, state)
    t_mixed = reduce_max(dist, mixed["elapsed_ms"])
    t_plain = reduce_max(dist, plain["elapsed_ms"])
    value = ws * n * args.steps / (t_mixed / 1e3)
    plain_value = ws * n * args.steps / (t_plain / 1e3)
    errs = {f: rel_l2(mixed["fields"][f] - (20.0 if f == "T" else 0.0),
                      plain["fields"][f] - (20.0 if f == "T" else 0.0))
            for f in ("u", "pl_strain", "sigma_eq", "T", "reaction_force")}
    e2e_steps = max(args.steps, 100)
    e2e_v, h2d, d2h = (0.0, 0, 0) if args.no_e2e else run_e2e(sc, "mixed", e2e_steps, state, mlp)
    e2e_v = reduce_max(dist, e2e_v) * ws if dist else e2e_v

    peak, peak_kind = measured_peaks()
    dom = mixed["dominant"]
    per_launch_ms = mixed["kernel_ms"] / max(mixed["kernel_launches"], 1)
    alg_bytes = LAUNCH_BYTES_MIXED.get(dom, BYTES_MODEL["mixed"][dom]) * n
    if dom in PAIR_KERNELS:
        alg_bytes_idx = alg_bytes + NB_INDEX_BYTES * 56 * n
    else:
        alg_bytes_idx = alg_bytes
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        if dom in tj.get("mixed", {}):
            traffic = tj["mixed"][dom] * n
    step_bytes = sum(BYTES_MODEL["mixed"].values()) * n
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": warmup, "ms_per_step": t_mixed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": config,
        "plain_fp64": {"value": plain_value, "ms_per_step": t_plain / args.steps,
                       "dominant_kernel": plain["dominant"],
                       "per_kernel_ms": plain["per_kernel_ms"],
                       "newton_iters_per_plastic_particle": plain["newton_iters_per_call"]},
        "speedup_vs_plain_fp64": value / plain_value,
        "rel_l2_vs_fp64": errs,
        "rel_l2_vs_fp64_note": "both forms restored from the same %d-step plastic state; "
                               "fields after the warm-up, profiled and timed steps (%d steps), "
                               "reaction_force = the platen's curve over 20 further steps"
                               % (args.preload, warmup + 5 * 20 + args.steps + 20),
        "mlp_warm_start": mlp is not None,
        "mlp": None if mlp is None else dict(
            mlp_info,
            used_per_step=mixed["mlp_used_per_step"],
            newton_iters_with_mlp=mixed["newton_iters_per_call"],
            newton_iters_without_mlp=mixed_nomlp["newton_iters_per_call"],
            mixed_without_mlp_ms_per_step=mixed_nomlp["elapsed_ms"] / args.steps),
        "newton_iters_per_plastic_particle": mixed["newton_iters_per_call"],
        "plastic_particles_per_step": mixed["plastic_per_step"],
        "plastic_fraction_at_start": state["_plastic_fraction"],
        "per_kernel_ms": mixed["per_kernel_ms"],
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "alg_bytes_per_launch": alg_bytes,
                     "alg_bytes_with_nb_index": alg_bytes_idx,
                     "achieved_with_nb_index": alg_bytes_idx / (per_launch_ms / 1e3) / 1e9,
                     "step_achieved_GBs": step_bytes / (t_mixed / args.steps / 1e3) / 1e9},
        "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                "note": "create + setters from pinned host arrays + solve + read-back into pinned host arrays + destroy, host clock; median of 3 calls after 1 warm-up call"},
        "gpu_launches": mixed["launches"],
        "clocks": mixed["clocks"],
    }
    if not args.no_extra and rank == 0:
        line["rel_l2_vs_fp64_from_rest"] = from_rest_errors(mlp, args.from_rest_steps)
        line["fp64_ceiling"] = fp64_ceiling(plain["per_kernel_ms"], n)
        line["heat"] = bench_heat(args)
        line["indentation"] = bench_indentation(args)
    if rank == 0:
        line["cpu_baseline"] = None if args.no_cpu else cpu_baseline(sc)
        print(json.dumps(line))


if __name__ == "__main__":
    main()
