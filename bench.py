"""Benchmark of the per-step SPH + Barnes-Hut gravity hot path on GB300.

Workload (the mixed-precision configuration of the headline metric): a basalt target of 1,000,000
requested HCP particles (R = 50 km) hit by a 20,000-particle impactor (R = 5 km) at 5 km/s and 45 degrees;
Hooke + von Mises + Grady-Kipp damage, SolidStressForce + StandardAV, adaptive h, Barnes-Hut theta = 0.5
octupole, predictor-corrector with the Courant criterion. One step is one ITimeStepping::step over the whole
particle set. The state (~300 B per particle) exceeds the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0). `value` is the mixed-precision path with the state resident in HBM; `e2e`
is the same metric through the public API with host buffers (positions and velocities uploaded from pinned
host memory and positions, velocities, density and energy read back every step); `fp64` reports the plain
FP64 GPU path on the same workload, the mixed path's error against it after 100 steps (fields and conserved
totals) and both paths' error against the CPU oracle after the first steps; `nbody_plummer` the 4,194,304-
particle Plummer walk at theta 0.3 / 0.5 / 0.7 against the FP64 direct sum on 65,536 particles; `fp64_configs`
the FP64 GPU path against the CPU oracle on the 10,648-particle sphere and the 217,823-particle impact;
`adjoint` and `nbody_reaccumulation` the adjoint and N-body workloads. `roofline` divides by the FP32 rate
measured on the device in the same run. `--impl reference` times the CPU implementation of the path (the
oracle restatement of the reference, all host threads) on the same workload.
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

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "particle-steps/s (1M SPH+gravity): mixed vs FP64 GPU at stated err; adjoint/fwd"
UNIT = "particle-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--n-target", type=int, default=1_000_000)
    ap.add_argument("--n-impactor", type=int, default=20_000)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--error-steps", type=int, default=100,
                    help="steps after which the mixed path is compared with the FP64 GPU path")
    ap.add_argument("--port-error-steps", type=int, default=5,
                    help="steps after which both GPU paths are compared with the CPU oracle (0: skip)")
    ap.add_argument("--no-fp64-configs", action="store_true",
                    help="skip the FP64 GPU vs CPU lines of the 10,648- and 217,823-particle configurations")
    ap.add_argument("--profile-only", action="store_true", help="warm-up + timed steps only (for ncu)")
    ap.add_argument("--no-nbody", action="store_true", help="skip the gravity-only Plummer measurement")
    ap.add_argument("--nbody-n", type=int, default=4_194_304)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement")
    ap.add_argument("--no-reaccumulation", action="store_true", help="skip the N-body collision measurement")
    ap.add_argument("--reacc-n", type=int, default=1_000_000)
    ap.add_argument("--only", choices=["nbody", "adjoint", "reaccumulation", "fp64_configs"], default=None,
                    help="run only one of the secondary measurements and print its JSON (for profiling)")
    ap.add_argument("--adjoint-target", type=int, default=100_000)
    ap.add_argument("--adjoint-impactor", type=int, default=2_000)
    return ap.parse_args()


def workload(args):
    from opensph_gb300 import abi, initial

    st, mats = initial.impact_state(args.n_target, 5.0e4, args.n_impactor, 5.0e3, speed=5.0e3, angle_deg=45.0,
                                    seed=1234)
    n = len(st["m"])
    return st, mats, n


def make_config(n, mats, precision):
    from opensph_gb300 import abi

    return abi.make_config(n, mats, forces=abi.FORCE_PRESSURE | abi.FORCE_SOLID_STRESS | abi.FORCE_SELF_GRAVITY,
                           adaptive_h=True, precision=precision, initial_timestep=0.03)


def config_json(args, n):
    return {"workload": f"solid impact: basalt target {args.n_target} HCP requested (R 50 km) + impactor "
                        f"{args.n_impactor} (R 5 km) at 5 km/s, 45 deg; von Mises + Grady-Kipp, adaptive h, "
                        f"BH theta 0.5 octupole, predictor-corrector + Courant",
            "particles": n, "precision": "mixed (FP32 pair sums, FP64 state/integrator)",
            "l2": "state larger than L2 (no flush)", "parallelism": "replicas"}


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# algorithmic bytes per particle of the pair-loop kernel of this workload (solid physics, mixed inputs):
# reads the particle's own packed inputs (4 x float4 = 64 B, S/rho^2 5 x 4 B, FP64 r, rho, p, S for the
# finalize 32 + 16 + 40 B, agrav 32 B, flaw data eps_min, m_zero, growth, n_flaws, D 36 B, mat 4 B) = 244 B;
# writes dv 32, du, drho, divv 24, ncnt 4, gradv 48, dS 40, dD 8, v.h 8 = 164 B. Neighbour data are
# re-read from cache, not counted.
PAIR_BYTES_PER_PARTICLE = 244 + 164


def run_gpu(args, rank, world):
    import torch

    from opensph_gb300 import abi, replicas
    from opensph_gb300.solver import GpuSolver

    dev = replicas.world_info()[2]
    torch.cuda.set_device(dev)
    st, mats, n = workload(args)
    cfg, keep = make_config(n, mats, abi.PRECISION_MIXED)
    cfg.device = dev
    g = GpuSolver(cfg, keep)
    g.set_state(st)
    stream = torch.cuda.ExternalStream(g.stream)
    g.step(args.warmup)
    g.synchronize()
    if args.profile_only:
        g.step(args.steps)
        g.synchronize()
        return None
    g.set_profiling(True)
    g.phase_times()
    replicas.barrier()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        start.record(stream)
        g.step(args.steps)
        end.record(stream)
        end.synchronize()
    torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    phases, launches = g.phase_times()
    g.set_profiling(False)
    ms = replicas.max_over_ranks(ms, f"cuda:{dev}")
    value = replicas.job_rate(n, args.steps, world, ms)

    # end-to-end through the public API with host buffers
    pinned = {k: torch.empty(4 * n, dtype=torch.float64, pin_memory=True) for k in ("r", "v")}
    outs = {k: torch.empty(sz, dtype=torch.float64, pin_memory=True) for k, sz in
            (("r", 4 * n), ("v", 4 * n), ("rho", n), ("u", n))}
    state_now = g.get_state(["r", "v"])
    pinned["r"].numpy()[:] = state_now["r"]
    pinned["v"].numpy()[:] = state_now["v"]
    lib, hnd = g._lib, g._h
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_start = torch.cuda.Event(enable_timing=True)
    e2e_end = torch.cuda.Event(enable_timing=True)
    e2e_start.record(stream)
    for _ in range(args.steps):
        g._check(lib.sphgpu_set_quantity(hnd, abi.Q_POSITION, 0, pinned["r"].data_ptr(), n))
        g._check(lib.sphgpu_set_quantity(hnd, abi.Q_POSITION, 1, pinned["v"].data_ptr(), n))
        g.step(1)
        g._check(lib.sphgpu_get_quantity(hnd, abi.Q_POSITION, 0, outs["r"].data_ptr(), n))
        g._check(lib.sphgpu_get_quantity(hnd, abi.Q_POSITION, 1, outs["v"].data_ptr(), n))
        g._check(lib.sphgpu_get_quantity(hnd, abi.Q_DENSITY, 0, outs["rho"].data_ptr(), n))
        g._check(lib.sphgpu_get_quantity(hnd, abi.Q_ENERGY, 0, outs["u"].data_ptr(), n))
        # the state read back is the next step's input (the pinned buffers swap roles)
        pinned["r"], outs["r"] = outs["r"], pinned["r"]
        pinned["v"], outs["v"] = outs["v"], pinned["v"]
    e2e_end.record(stream)
    e2e_end.synchronize()
    e2e_wall = time.perf_counter() - t0
    e2e_ms = max(e2e_start.elapsed_time(e2e_end), e2e_wall * 1e3)
    e2e_value = replicas.job_rate(n, args.steps, world, replicas.max_over_ranks(e2e_ms, f"cuda:{dev}"))
    interactions = g.gravity_interactions()
    g.close()

    result = {"n": n, "ms": ms, "value": value, "phases": phases, "launches": launches, "interactions": interactions,
              "clocks": clk.summary(), "e2e": {"value": e2e_value, "unit": UNIT,
                                                 "h2d_bytes_per_step": 2 * 32 * n,
                                                 "d2h_bytes_per_step": (32 + 32 + 8 + 8) * n}}
    if rank == 0 and not args.no_fp64:
        result["fp64"] = compare_fp64(args, st, mats, n, cfg, dev)
    if rank == 0 and not args.no_nbody:
        result["nbody"] = nbody(args, dev)
    if rank == 0 and not args.no_adjoint:
        result["adjoint"] = adjoint(args, dev)
    if rank == 0 and not args.no_reaccumulation:
        result["reaccumulation"] = reaccumulation(args, dev)
    if rank == 0 and not args.no_fp64_configs:
        result["fp64_configs"] = fp64_configs(args, dev)
    if rank == 0:
        from opensph_gb300.solver import measure_fp32_peak

        result["fp32_peak_tflops"] = measure_fp32_peak(200.0)
    return result


def compare_fp64(args, st, mats, n, mixed_cfg, dev):
    """Plain FP64 GPU path on the same workload: speed, and the mixed path's error against it."""
    import torch

    from opensph_gb300 import abi
    from opensph_gb300.solver import GpuSolver

    from oracle import oracle

    steps = max(args.error_steps, args.warmup + args.steps)
    port_steps = args.port_error_steps
    out = {}
    states, totals, early = {}, {}, {}
    for name, prec in (("fp64", abi.PRECISION_FP64), ("mixed", abi.PRECISION_MIXED)):
        cfg, keep = make_config(n, mats, prec)
        cfg.device = dev
        with GpuSolver(cfg, keep) as g:
            g.set_state({k: v.copy() for k, v in st.items()})
            stream = torch.cuda.ExternalStream(g.stream)
            if port_steps > 0:
                g.step(port_steps)
                early[name] = g.get_state(["r", "v", "rho", "u"])
            if name == "fp64":
                g.step(args.warmup)
                s0 = torch.cuda.Event(enable_timing=True)
                s1 = torch.cuda.Event(enable_timing=True)
                s0.record(stream)
                g.step(args.steps)
                s1.record(stream)
                s1.synchronize()
                out["value"] = n * args.steps / (s0.elapsed_time(s1) * 1e-3)
                out["ms_per_step"] = s0.elapsed_time(s1) / args.steps
                g.step(steps - port_steps - args.warmup - args.steps)
            else:
                g.step(steps - port_steps)
            states[name] = g.get_state(["r", "v", "rho", "u", "D"])
            totals[name] = g.totals()
            out[f"{name}_final_timestep"] = g.timestep
    ref, mix = states["fp64"], states["mixed"]

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))

    vref = ref["v"].reshape(-1, 4)[:, :3]
    vmix = mix["v"].reshape(-1, 4)[:, :3]
    out["steps_compared"] = steps
    out["rel_err_density"] = rel(mix["rho"], ref["rho"])
    out["rel_err_velocity"] = rel(vmix, vref)
    out["rel_err_energy"] = rel(mix["u"], ref["u"])
    out["max_abs_err_damage"] = float(np.max(np.abs(mix["D"] - ref["D"])))
    # conserved totals (core/physics/Integrals.cpp:24-91) after the same steps: total energy relative to itself,
    # momentum and angular momentum relative to their largest component
    tm, tf = totals["mixed"], totals["fp64"]
    out["totals_after_steps"] = {
        "rel_err_total_energy": abs((tm[6] + tm[7]) - (tf[6] + tf[7])) / abs(tf[6] + tf[7]),
        "rel_err_momentum": float(np.max(np.abs(tm[0:3] - tf[0:3])) / np.max(np.abs(tf[0:3]))),
        "rel_err_angular_momentum": float(np.max(np.abs(tm[3:6] - tf[3:6])) / np.max(np.abs(tf[3:6]))),
        "fp64_total_energy": float(tf[6] + tf[7]), "fp64_momentum": [float(x) for x in tf[0:3]]}
    if port_steps > 0:
        # both GPU paths against the CPU implementation of the reference's algorithms (the oracle, all host
        # threads) after the first port_steps steps from the same state
        work = {k: v.copy() for k, v in st.items()}
        cfg64, _ = make_config(n, mats, abi.PRECISION_FP64)
        oracle.set_threads(0)
        oracle.run(cfg64, work, port_steps, float(cfg64.initial_timestep))
        vport = work["v"].reshape(-1, 4)[:, :3]
        port = {"steps": port_steps}
        for name in ("fp64", "mixed"):
            e = early[name]
            port[name] = {"rel_err_density": rel(e["rho"], work["rho"]),
                          "rel_err_velocity": rel(e["v"].reshape(-1, 4)[:, :3], vport),
                          "rel_err_energy": rel(e["u"], work["u"]),
                          "rel_err_position": rel(e["r"].reshape(-1, 4)[:, :3], work["r"].reshape(-1, 4)[:, :3])}
        out["vs_cpu_port"] = port
    return out


# DRAM bytes (read + write) of one launch of the walk's evaluation kernel on the default workload: a constant from
# a separate ncu capture of the same workload and command (dram__bytes_read.sum + dram__bytes_write.sum, caches
# flushed before the launch), not measured in this run
WALK_TRAFFIC_BYTES = (240.2 + 27.7) * 1e6
WALK_TRAFFIC_SOURCE = ("constant from an ncu capture of the evaluation kernel of one walk of this workload "
                       "(dram__bytes_read.sum + dram__bytes_write.sum, caches flushed before the launch); not "
                       "measured in this run")

# FP32 operations of one particle-multipole evaluation (accMultipoleF, csrc/gravity32.cu: octupole) and the
# N-body convention for one softened particle-particle interaction
FLOP_PN = 120
FLOP_PP = 20
FP32_PEAK_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12  # TFLOP/s at the maximum SM clock


def nbody(args, dev):
    """Gravity-only workload: Plummer sphere (scale radius 1, M = 1, G = 1, softening 1e-3 as h), 4,194,304
    particles, Barnes-Hut octupole at theta 0.3, 0.5 and 0.7: tree build + walk timed for the mixed (FP32
    evaluation) and the FP64 walk; both checked against the FP64 direct sum (BruteForceGravity,
    sphgpu_gravity_direct) on 65,536 seeded particles."""
    import torch

    from opensph_gb300 import abi, initial
    from opensph_gb300.solver import GpuSolver

    n = args.nbody_n
    r, m = initial.plummer(n, seed=7, softening=1e-3)
    r = r.ravel()
    targets = np.sort(np.random.default_rng(11).choice(n, size=min(65536, n), replace=False)).astype("u4")
    out = {"particles": n, "workload": "Plummer sphere, G = 1, softening 1e-3, octupole",
           "direct_check_targets": int(targets.size)}

    def solver(theta, prec):
        cfg, keep = abi.make_config(n, [abi.ideal_gas()], forces=abi.FORCE_PRESSURE | abi.FORCE_SELF_GRAVITY,
                                    gravity_constant=1.0, gravity_opening_angle=theta, precision=prec)
        cfg.device = dev
        g = GpuSolver(cfg, keep)
        g.set_quantity(abi.Q_POSITION, 0, r)
        g.set_quantity(abi.Q_MASS, 0, m)
        return g

    t0 = time.perf_counter()
    with solver(0.5, abi.PRECISION_FP64) as g:
        direct = g.gravity_direct(targets).reshape(-1, 4)[:, :3]
    out["direct_sum_s"] = time.perf_counter() - t0
    dnorm = np.linalg.norm(direct, axis=1)

    def errors(acc):
        e = np.linalg.norm(acc.reshape(-1, 4)[targets, :3] - direct, axis=1) / dnorm
        return {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)), "max": float(np.max(e))}

    for theta in (0.3, 0.5, 0.7):
        res = {}
        accs = {}
        for name, prec in (("mixed", abi.PRECISION_MIXED), ("fp64", abi.PRECISION_FP64)):
            with solver(theta, prec) as g:
                g.gravity()
                g.set_profiling(True)
                g.phase_times()
                reps = 3 if name == "mixed" else 1
                for _ in range(reps):
                    accs[name] = g.gravity()
                phases, _ = g.phase_times()
                inter = g.gravity_interactions()
            walk_ms = phases["gravity_eval"] / reps
            build_ms = phases["gravity_build"] / reps
            total = inter[0] + inter[1]
            flops = inter[0] * FLOP_PN + inter[1] * FLOP_PP
            res[name] = {"walk_ms": walk_ms, "build_ms": build_ms, "interactions": total,
                         "particle_node": inter[0], "particle_particle": inter[1],
                         "interactions_per_s": total / (walk_ms * 1e-3),
                         "walk_tflops": flops / (walk_ms * 1e-3) / 1e12,
                         "rel_err_vs_direct": errors(accs[name])}
        res["walk_speedup_mixed_vs_fp64"] = res["fp64"]["walk_ms"] / res["mixed"]["walk_ms"]
        a, b = accs["mixed"].reshape(-1, 4)[:, :3], accs["fp64"].reshape(-1, 4)[:, :3]
        res["mixed_vs_fp64_rel_err"] = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
        out[f"theta_{theta}"] = res
    torch.cuda.synchronize()
    return out


def fp64_configs(args, dev):
    """The plain FP64 path on the two CPU-runnable configurations, GPU against the CPU implementation of the
    reference's algorithms (the oracle, all host threads), same inputs:
    config 1, the basalt sphere of 10,000 requested particles (HCP, R = 10 km, h = 1.3 x the lattice spacing,
    rho 2700, u 1e3, velocities N(0, 1 m/s) per component), Tillotson, continuity + pressure + standard AV,
    Barnes-Hut theta 0.5 octupole, predictor-corrector with the Courant criterion, 100 steps;
    config 2, the solid impact of 200,000 + 5,000 requested particles (R 50 km and 5 km, 5 km/s at 45 degrees),
    von Mises + Grady-Kipp, adaptive h."""
    import torch

    from opensph_gb300 import abi, initial
    from opensph_gb300.solver import GpuSolver
    from oracle import oracle

    out = {}
    # config 1
    rr = initial.hcp_sphere(10000, 1.0e4, eta=1.43)
    n1 = len(rr)
    volume = 4.0 / 3.0 * np.pi * 1.0e12
    vel = np.zeros((n1, 4))
    vel[:, :3] = np.random.default_rng(1).standard_normal((n1, 3))
    st1 = {"r": rr.ravel(), "v": vel.ravel(), "dv": np.zeros(4 * n1), "m": np.full(n1, 2700.0 * volume / n1),
           "rho": np.full(n1, 2700.0), "drho": np.zeros(n1), "u": np.full(n1, 1.0e3), "du": np.zeros(n1),
           "p": np.zeros(n1), "cs": np.zeros(n1), "divv": np.zeros(n1), "ncnt": np.zeros(n1, "u4"),
           "flag": np.zeros(n1, "u4"), "mat": np.zeros(n1, "u4")}
    mat1 = abi.basalt(yielding=abi.YIELDING_NONE, damage=abi.DAMAGE_NONE)
    cfg1, keep1 = abi.make_config(n1, [mat1], forces=abi.FORCE_PRESSURE | abi.FORCE_SELF_GRAVITY)
    # config 2
    st2, mats2 = initial.impact_state(200000, 5.0e4, 5000, 5.0e3, speed=5.0e3, angle_deg=45.0, seed=1234)
    n2 = len(st2["m"])
    cfg2, keep2 = make_config(n2, mats2, abi.PRECISION_FP64)
    for name, st, cfg, gpu_steps, cpu_steps in (("config1_sphere", st1, cfg1, 100, 100),
                                                ("config2_impact", st2, cfg2, 20, 2)):
        cfg.device = dev
        with GpuSolver(cfg, [keep1, keep2]) as g:
            g.set_state({k: v.copy() for k, v in st.items()})
            g.step(3)
            g.synchronize()
            stream = torch.cuda.ExternalStream(g.stream)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.step(gpu_steps)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
        work = {k: v.copy() for k, v in st.items()}
        oracle.set_threads(0)
        t0 = time.perf_counter()
        oracle.run(cfg, work, cpu_steps, float(cfg.initial_timestep))
        secs = time.perf_counter() - t0
        n = len(st["m"])
        gpu = n * gpu_steps / (ms * 1e-3)
        cpu = n * cpu_steps / secs
        out[name] = {"particles": n, "fp64_gpu": {"value": gpu, "unit": UNIT, "ms_per_step": ms / gpu_steps,
                                                 "steps": gpu_steps},
                     "cpu": {"value": cpu, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                             "steps": cpu_steps, "seconds": secs},
                     "gpu_over_cpu": gpu / cpu}
    return out


def reaccumulation(args, dev):
    """N-body workload (HardSphereSolver, the reaccumulation phase of the reference's impact presets): a cloud of
    hard spheres (radius 400-600 m, density 2500, radius 140 km for 1M spheres, inflow 2e-4 r plus a 0.1 m/s
    dispersion), the N-body run's settings (leap-frog, acceleration criterion, BH theta 0.8 with solid spheres,
    merge-or-bounce collisions, pass-or-merge overlaps), max step 100 s. Mixed-precision walk; collisions in
    FP64. Timed K steps after W warm-up steps; CPU baseline: one step of the oracle on all host cores."""
    import torch

    from opensph_gb300 import abi, initial
    from opensph_gb300.solver import GpuSolver
    from oracle import oracle

    n = args.reacc_n
    radius = 140000.0 * (n / 1.0e6) ** (1.0 / 3.0)
    st = initial.rubble_cloud(n, radius, inflow=2e-4, sigma=0.1)
    cfg, keep = abi.make_nbody_config(n, max_timestep=100.0, initial_timestep=100.0, precision=abi.PRECISION_MIXED)
    cfg.device = dev
    with GpuSolver(cfg, keep) as g:
        g.set_state(st)
        g.step(args.warmup)
        g.synchronize()
        stats0 = g.collision_stats()
        g.set_profiling(True)
        g.phase_times()
        prof0 = g.collision_profile()
        stream = torch.cuda.ExternalStream(g.stream)
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        g.step(args.steps)
        end.record(stream)
        end.synchronize()
        ms = start.elapsed_time(end)
        phases, launches = g.phase_times()
        stats1 = g.collision_stats()
        prof1 = g.collision_profile()
        n_end = g.n
        dt_end = g.timestep
    events = [(b - a) / args.steps for a, b in zip(stats0, stats1)]
    out = {"particles": n, "particles_after": n_end, "workload": "rubble cloud, N-body with collisions",
           "ms_per_step": ms / args.steps, "value": n * args.steps / (ms * 1e-3), "unit": UNIT,
           "events_per_step": {"collisions": events[0], "mergers": events[1], "bounces": events[2],
                               "overlaps": events[3]},
           "phases_ms_per_step": {k: v / args.steps for k, v in phases.items() if v > 0},
           "gpu_launches": launches, "timestep_after": dt_end}
    # SM cycles of the collision loop per processed record: serial part (selection, handler, invalidation),
    # re-searches, insertion of the new records (sphgpu_collision_profile)
    rec = prof1[0] - prof0[0]
    if rec > 0:
        out["collision_loop"] = {"records": rec, "cycles_per_record": {
            "serial": (prof1[1] - prof0[1]) / rec, "research": (prof1[2] - prof0[2]) / rec,
            "insert": (prof1[3] - prof0[3]) / rec}}
    if not args.no_cpu:
        work = initial.rubble_cloud(n, radius, inflow=2e-4, sigma=0.1)
        cfg64, keep64 = abi.make_nbody_config(n, max_timestep=100.0, initial_timestep=100.0)
        oracle.set_threads(0)
        t0 = time.perf_counter()
        oracle.nbody_run(cfg64, work, 1, 100.0)
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / secs, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"1 step of the {n}-particle cloud from its initial state ({secs:.1f} s, "
                                         "FP64 oracle, gravity on all host threads, collisions sequential after "
                                         "a parallel first pass)"}
    return out


ADJ_STEPS = 50
ADJ_DT = 1.0e-3
ADJ_REBUILD = 10
ADJ_CHECKPOINT = 10


def adjoint(args, dev):
    """Adjoint workload: ideal-gas sphere (rho 1, p 1) + impactor at Mach 3, 50 leap-frog steps of continuity +
    pressure + standard AV over lists rebuilt every 10 steps, checkpoints every 10 steps, loss = sum |v_target|^2.
    Times sphgpu_adjoint_forward and sphgpu_adjoint_backward (host wall clock around each call, which ends with
    the results on the host) in FP64 and mixed precision, and checks each gradient against FP64 central finite
    differences (the FP64 forward, eps 1e-7) in 8 seeded smooth directions of all positions, the impactor
    velocity and the AV alpha."""
    from opensph_gb300 import abi, initial
    from opensph_gb300.solver import GpuSolver

    st, nt = initial.gas_impact(args.adjoint_target, args.adjoint_impactor)
    n = len(st["m"])
    pos = st["r"].reshape(-1, 4)[:, :3]

    def solver(state):
        cfg, keep = abi.make_config(n, [abi.ideal_gas()], forces=abi.FORCE_PRESSURE)
        cfg.device = dev
        g = GpuSolver(cfg, keep)
        g.set_state({k: state[k] for k in ("r", "v", "m", "rho", "u")})
        return g

    def acfg(prec, alpha=1.5):
        return abi.make_adjoint_config(ADJ_STEPS, ADJ_DT, nt, rebuild_every=ADJ_REBUILD,
                                       checkpoint_every=ADJ_CHECKPOINT, alpha=alpha, precision=prec)

    out = {"particles": n, "targets": nt, "steps": ADJ_STEPS, "dt": ADJ_DT, "rebuild_every": ADJ_REBUILD,
           "checkpoint_every": ADJ_CHECKPOINT,
           "workload": f"ideal gas (gamma 5/3) sphere {nt} + impactor {n - nt} at Mach 3, contracting at 5% c_s; "
                       "continuity + pressure + standard AV, leap-frog, frozen lists; loss = sum |v_target|^2"}
    grads = {}
    for name, prec in (("fp64", abi.PRECISION_FP64), ("mixed", abi.PRECISION_MIXED)):
        with solver(st) as g:
            g.adjoint_forward(acfg(prec))  # warm-up (allocation, list capacity)
            g.adjoint_backward()
            fw, bw = [], []
            for _ in range(3):
                t0 = time.perf_counter()
                loss = g.adjoint_forward(acfg(prec))
                t1 = time.perf_counter()
                grads[name] = g.adjoint_backward()
                t2 = time.perf_counter()
                fw.append(t1 - t0)
                bw.append(t2 - t1)
        f, b = min(fw) * 1e3, min(bw) * 1e3
        out[name] = {"loss": loss, "forward_ms": f, "backward_ms": b, "forward_ms_per_step": f / ADJ_STEPS,
                     "backward_ms_per_step": b / ADJ_STEPS, "adjoint_over_forward": b / f}
    rng = np.random.default_rng(5)
    # 1e-7: small enough that few pair terms cross a kink of the model (kernel-table nodes, the AV switch,
    # list membership) between the two evaluations, large enough for the FP64 loss's rounding
    eps = 1e-7
    errs = {"fp64": 0.0, "mixed": 0.0}
    for _ in range(8):
        dr = np.zeros((n, 4))
        for _m in range(3):
            k = 2.0 * rng.standard_normal(3)
            ph = 2.0 * np.pi * rng.random()
            amp = rng.standard_normal(3)
            dr[:, :3] += np.sin(pos @ k + ph)[:, None] * amp[None, :]
        dv = np.zeros((n, 4))
        dv[nt:, :3] = rng.standard_normal(3)
        da = float(rng.standard_normal())
        vals = []
        for sgn in (1.0, -1.0):
            sp = dict(st)
            sp["r"] = st["r"] + sgn * eps * dr.ravel()
            sp["v"] = st["v"] + sgn * eps * dv.ravel()
            with solver(sp) as g:
                vals.append(g.adjoint_forward(acfg(abi.PRECISION_FP64, 1.5 + sgn * eps * da)))
        fd = (vals[0] - vals[1]) / (2 * eps)
        for name, gr in grads.items():
            mine = float(np.dot(gr["r"], dr.ravel()) + np.dot(gr["v"], dv.ravel())) + gr["alpha"] * da
            errs[name] = max(errs[name], abs(mine - fd) / abs(fd))
    for name in errs:
        out[name]["fd_max_rel_err_8_directions"] = errs[name]
    out["mixed_vs_fp64_loss_rel_err"] = abs(out["mixed"]["loss"] - out["fp64"]["loss"]) / abs(out["fp64"]["loss"])
    return out


def cpu_sample(args, st, mats, n, steps):
    """The CPU implementation (oracle restatement of the reference, all host threads) on the same state."""
    from opensph_gb300 import abi
    from oracle import oracle

    cfg, keep = make_config(n, mats, abi.PRECISION_FP64)
    work = {k: v.copy() for k, v in st.items()}
    oracle.set_threads(0)
    t0 = time.perf_counter()
    oracle.run(cfg, work, steps, 0.03)
    dt = time.perf_counter() - t0
    return n * steps / dt, dt


def main():
    args = parse()
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        st, mats, n = workload(args)
        cores = os.cpu_count() or 1
        steps = args.warmup + args.steps
        value, secs = cpu_sample(args, st, mats, n, steps)
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": config_json(args, n),
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": f"{steps} full steps of the {n}-particle workload (FP64 oracle)"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    import torch

    if args.only is not None:
        dev = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(dev)
        out = {"nbody": nbody, "adjoint": adjoint, "reaccumulation": reaccumulation,
               "fp64_configs": fp64_configs}[args.only](args, dev)
        print(json.dumps({args.only: out}))
        return

    if world > 1:
        torch.distributed.init_process_group("nccl")
    res = run_gpu(args, rank, world)
    if res is None or rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    n = res["n"]
    ms_step = res["ms"] / args.steps
    pair_ms = res["phases"]["sph_eval"] / args.steps
    peak, peak_kind = peaks()
    achieved = PAIR_BYTES_PER_PARTICLE * n / (pair_ms * 1e-3) / 1e9 if pair_ms > 0 else None
    # dominant kernel: the mixed tree walk's evaluation kernel, FP32-pipe bound; algorithmic FLOPs of the last
    # step's walk (interaction counts of the walk itself) over the kernel's CUDA-event time on the gravity stream
    # (the whole walk, with its interaction-list phase, beside it)
    eval_ms = res["phases"]["walk_evaluation"] / args.steps
    walk_ms = res["phases"]["gravity_eval"] / args.steps
    pn, pp = res["interactions"]
    walk_flops = pn * FLOP_PN + pp * FLOP_PP
    walk_tf = walk_flops / (eval_ms * 1e-3) / 1e12 if eval_ms > 0 else None
    whole_tf = walk_flops / (walk_ms * 1e-3) / 1e12 if walk_ms > 0 else None
    fp32_peak = res.get("fp32_peak_tflops") or FP32_PEAK_NOMINAL
    fp32_source = ("measured: FMA-chain kernel on every SM, CUDA events (sphgpu_measure_fp32_peak)"
                   if res.get("fp32_peak_tflops") else "nominal (152 SMs x 128 lanes x 2 x 2.07 GHz)")
    line = {
        "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic", "config": config_json(args, n),
        "e2e": res["e2e"], "gpu_launches": res["launches"], "clocks": res["clocks"],
        "phases_ms_per_step": {k: v / args.steps for k, v in res["phases"].items()},
        "roofline": {"kernel": "evalListsKernel (mixed walk evaluation)", "bound": "fp32", "achieved": walk_tf,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": walk_tf / fp32_peak if walk_tf else None,
                     "traffic": WALK_TRAFFIC_BYTES, "traffic_source": WALK_TRAFFIC_SOURCE,
                     "peak_source": fp32_source, "fp32_nominal_tflops": FP32_PEAK_NOMINAL,
                     "flops_per_launch": walk_flops, "particle_node": pn, "particle_particle": pp,
                     "flop_per_particle_node": FLOP_PN, "flop_per_particle_particle": FLOP_PP,
                     "launch_ms": eval_ms, "whole_walk_ms": walk_ms, "whole_walk_achieved": whole_tf,
                     "whole_walk_frac": whole_tf / fp32_peak if whole_tf else None},
        "roofline_pair": {"kernel": "pairSumMixedKernel", "bound": "hbm", "achieved": achieved, "peak": peak,
                          "unit": "GB/s", "frac": achieved / peak if achieved else None,
                          "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                          "algorithmic_bytes_per_particle": PAIR_BYTES_PER_PARTICLE,
                          "note": "timed from its queueing to its end, beside the tree's moments and walk on the "
                                  "gravity stream"},
    }
    if "fp64" in res:
        line["fp64"] = res["fp64"]
    if "nbody" in res:
        line["nbody_plummer"] = res["nbody"]
    if "adjoint" in res:
        line["adjoint"] = res["adjoint"]
    if "reaccumulation" in res:
        line["nbody_reaccumulation"] = res["reaccumulation"]
    if "fp64_configs" in res:
        line["fp64_configs"] = res["fp64_configs"]
    if not args.no_cpu:
        st, mats, n2 = workload(args)
        value, secs = cpu_sample(args, st, mats, n2, args.cpu_steps)
        line["cpu_baseline"] = {"value": value, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"{args.cpu_steps} full step(s) of the {n2}-particle workload "
                                          f"({secs:.1f} s, FP64 oracle, all host threads)"}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
