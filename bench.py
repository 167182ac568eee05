"""Benchmark of the GB300 Rigid IPC narrow phase.

One step = one narrow-phase pass of a Newton iteration on the large plain
scene (1000 subdivision-3 icospheres, radii U[0.3, 0.6] m, over a static
floor; dhat = 1e-3, dt = 0.01): continuous hash-grid broad phase between the
current poses and the poses after one explicit step of the seeded velocities
(v ~ N(0, 1), omega ~ N(0, 2)), rigid interval CCD over every candidate,
discrete broad phase at the current poses, constraint set, barrier energy,
gradient and PSD-projected 12x12 pair Hessians, and the block-sparse
assembly.  The poses are a seeded contact-rich pile (bounding-sphere
relaxation, 2e-4 m gaps) standing in for the settled state of that scene.

value: candidate pairs per second = (continuous candidates through the CCD
+ discrete candidates through the constraint set / barrier) / step time, with
inputs resident in HBM; e2e: the same through rigc_narrow_phase_host from
host buffers (pose upload and gradient / Hessian download inside the timed
region).  L2 is flushed (a 512 MiB write) before every timed step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "rigid-ipc_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "candidate pairs/s (CCD+barrier grad/Hess)"
UNIT = "pairs/s"
CCD_BYTES_PER_PAIR = 304        # ids + 4 rest vertices + 4 poses + toi
# DRAM bytes (read + write) per continuous candidate of one CCD call (all its
# search launches and the splits of their deferred pieces), from ncu captures
# of the 200-icosphere pile (132,242 candidates): k_ccd 56.95 MB read +
# 311.51 MB written over two launches (per-lane candidate state spilling
# from L1, the frame cache; it searches without time windows);
# k_ccd_group<32, 4> (one search per warp fitted to 4 blocks per SM)
# 119.20 MB + 40.87 MB and k_ccd_group<16, 4> (one search per half-warp, the
# same fit) 134.27 MB + 32.55 MB over three launches with time windows from
# 2^-6, most of it the deferred pieces written and read back and the spills.
# The traffic of a full call is this times its candidates.  FP64 figures of
# the first launch of the same calls: pipe active (fraction of peak) and
# lane-level GFLOP/s (dadd + dmul + 2 dfma over the launch).
K_CCD_DRAM_BYTES_PER_CANDIDATE = {
    "k_ccd": (42209536 + 14743808 + 310226176 + 1279232) / 132242,
    "k_ccd_group<32, 4>": (119197184 + 40870912) / 132242,
    "k_ccd_group<16, 4>": (134271488 + 32547072) / 132242}
K_CCD_FP64 = {"k_ccd": {"pipe_active": 0.233, "lane_gflops": 53.0},
              "k_ccd_group<32, 4>": {"pipe_active": 0.416, "lane_gflops": 108.6},
              "k_ccd_group<16, 4>": {"pipe_active": 0.343, "lane_gflops": 73.5}}
BARRIER_BYTES_PER_CONSTRAINT = 1456
# the CCD kernel of each search mode (rigc_set_tune's ccd_warp)
CCD_KERNELS = {0: "k_ccd", 1: "k_ccd_group<32, 1>", 2: "k_ccd_group<32, 4>",
               3: "k_ccd_group<32, 5>", 4: "k_ccd_group<16, 1>", 5: "k_ccd_group<16, 4>"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="rigc", choices=["rigc", "reference"])
    ap.add_argument("--bodies", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sim", action="store_true", help="skip the steps/s measurement")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the built-in launch shapes for the headline pass")
    ap.add_argument("--ccd-warp", type=int, default=None,
                    help="CCD kernel variant for the headline pass instead of the autotuner's "
                         "(rigc_set_tune's ccd_warp: 0 per lane, 1 per warp, 2 / 3 per warp "
                         "fitted to 4 / 5 blocks per SM, 4 per half-warp, 5 per half-warp "
                         "fitted to 4 blocks per SM)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the per-configuration pass rates")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the differentiable rollout measurement")
    ap.add_argument("--no-pl", action="store_true",
                    help="skip the piecewise-linear trajectory CCD measurement")
    ap.add_argument("--no-barrier", action="store_true",
                    help="skip the barrier-terms-at-scale measurement (slab stacks)")
    ap.add_argument("--barrier-columns", type=int, default=4,
                    help="slab stacks of the barrier measurement: N x N columns of 2 slabs")
    ap.add_argument("--sim-steps", type=int, default=20)
    ap.add_argument("--batch-sim-steps", type=int, default=2,
                    help="timed steps of the batched time step (0 skips it)")
    ap.add_argument("--batch-sim-plain-sample", type=int, default=16,
                    help="scenes timed one context each for the plain steps/s")
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes of the batched-vs-plain measurement (0 skips it)")
    return ap.parse_args()


def make_workload(n_bodies, seed):
    from rigc import scene as S

    spec = S.spec_icospheres(seed=seed, n=n_bodies)
    sc = S.scene_from_json(spec)
    x0 = S.packed_pile_poses(sc, seed=seed)
    x1 = sc.predictor_poses(x0)
    return sc, x0, x1


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                 f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 4 + i and s[4 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def broad_phase_roofline(sc, n_pairs, t, peak, peak_kind):
    """The continuous broad phase against its algorithmic bytes: rest
    vertices read (24 B each), two poses per body (96 B), an interval box
    written per vertex, edge and face (48 B), a candidate pair written (8 B)."""
    nv, ne, nf, nb = sc.num_vertices, len(sc.edges), len(sc.faces), sc.num_bodies
    b = nv * 24 + nb * 96 + (nv + ne + nf) * 48 + n_pairs * 8
    achieved = b / t / 1e9
    return {"kernel": "continuous broad phase (all its launches)", "bound": "hbm",
            "algorithmic_bytes": b, "ms": t * 1e3, "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind}


def fp64_peak():
    """The device's FP64 issue rate measured by the library's own DFMA / DADD
    chains (rigc_fp64_throughput): all lanes of every warp, then 16 and 1
    active lanes per warp, which shows whether a warp instruction costs the
    FP64 unit the same time whatever its active lanes."""
    import rigc

    out = {}
    for op, lanes in (("dfma", 32), ("dfma", 16), ("dfma", 1), ("dadd", 32)):
        r = rigc.fp64_throughput(op, lanes, 4096)
        out[f"{op}_{lanes}"] = {"gflops": r["gflops"], "warp_inst_per_s": r["warp_inst_per_s"],
                                "ms": r["ms"]}
    return out


def fp64_roofline(captured, measured):
    """The CCD kernel's FP64 side: its pipe-active fraction and lane-level
    FP64 rate from the ncu capture, against the FP64 peak measured in this
    run (all-lane DFMA chains)."""
    if not captured:
        return None
    out = dict(captured, source="ncu capture of the 200-icosphere pile", nominal_gflops=1250.0)
    if measured:
        peak = measured["dfma_32"]["gflops"]
        out["measured_peak_gflops"] = peak
        out["frac_of_measured"] = captured["lane_gflops"] / peak
    return out


def pl_rate(ctx, sc, x0, x1, x0d, x1d, timed, with_cpu=True, sample=2000):
    """The piecewise-linear trajectory CCD (the reference's JSON default
    trajectory) over the headline's continuous candidates: one narrow-phase
    call, device-timed; the oracle on a seeded sample of the same candidates
    on every host core beside it."""
    ee, fv = ctx.detect_collision_candidates_rigid(x0d, x1d, True, 0.0)
    n = len(ee) + len(fv)
    t_pl = timed(lambda: ctx.earliest_toi_piecewise_linear(x0d, x1d), reps=1)
    st = ctx.stats()
    out = {"workload": "the headline pile's continuous candidates, trajectory PIECEWISE_LINEAR, "
                       "dmin 0, every candidate searched in full",
           "candidates": n, "ms": t_pl * 1e3, "pairs_per_s": n / t_pl,
           "linear_ccd_boxes": st["ccd_boxes"], "kernel": "k_pl_ccd (one candidate per warp)"}
    if with_cpu:
        import oracle as O

        O.build()
        o = O.OracleScene(sc)
        rng = np.random.default_rng(0)
        sel = rng.choice(n, size=min(sample, n), replace=False)
        e_s, f_s = ee[sel[sel < len(ee)]], fv[sel[sel >= len(ee)] - len(ee)]
        cores = os.cpu_count() or 1
        t = time.perf_counter()
        o.pl_earliest_toi(x0, x1, e_s, f_s, nthreads=cores)
        t = time.perf_counter() - t
        out["cpu_oracle_pairs_per_s"] = len(sel) / t
        out["cpu_oracle_cores"] = cores
        out["cpu_oracle_sample"] = f"{len(sel)} seeded candidates"
    return out


def cpu_pass(o, x0, x1, dhat, nthreads):
    """One narrow-phase pass of the oracle (a port of the reference's CPU
    path), the work of one bench step: continuous broad phase, CCD over every
    candidate, discrete broad phase, constraint set, barrier terms; its
    wall time in seconds."""
    t = time.perf_counter()
    ee, fv = o.detect_candidates(x0, x1, True, 0.0)
    o.earliest_toi(x0, x1, ee, fv, nthreads=nthreads)
    ee_d, fv_d = o.detect_candidates(x0, continuous=False, inflation=dhat / 2)
    cs = o.constraint_set(x0, ee_d, fv_d, dhat)
    o.barrier_term(x0, cs, dhat)
    return time.perf_counter() - t


CPU_SAMPLE = ("one whole narrow-phase pass per step: both hash-grid broad phases, the CCD over "
              "every candidate and the barrier terms on {n} threads, the constraint set on 1 thread")


def cpu_baseline(sc, x0, x1, dhat, passes=2):
    """The oracle's pass on every host core: the last of a few passes (the
    first one warms the caches)."""
    import oracle as O

    O.build()
    o = O.OracleScene(sc)
    nthreads = os.cpu_count() or 1
    ee, fv = o.detect_candidates(x0, x1, True, 0.0)
    ee_d, fv_d = o.detect_candidates(x0, continuous=False, inflation=dhat / 2)
    n = len(ee) + len(fv) + len(ee_d) + len(fv_d)
    t = min(cpu_pass(o, x0, x1, dhat, nthreads) for _ in range(passes))
    return {"pairs_per_s": n / t, "pass_s": t, "cores": nthreads,
            "sample": CPU_SAMPLE.format(n=nthreads)}


SIM_WORKLOAD = ("27 unit cubes in a 3x3x3 lattice (spacing 1.05 m, seeded rotations and "
                "velocities) over a static plane; dt 0.01, dhat 1e-3, g 9.81, implicit-Euler "
                "IPC Newton solve per step, friction off")


SIM_FIRST = 25  # steps before the timed window (the cubes reach the plane around step 30)


def sim_rate(args, torch):
    """Simulated steps per second of the device time step on the small plain
    scene over steps SIM_FIRST .. SIM_FIRST + sim_steps, and the oracle's
    restated CPU step over the same window (bounded in time) as its
    baseline."""
    import rigc
    from rigc import scene as S

    sc = S.scene_from_json(S.spec_cubes(args.seed))
    ctx = rigc.Context(sc)
    ctx.sim_init(0.01, (0.0, -9.81, 0.0), 1e-3)
    ctx.sim_step(SIM_FIRST)  # the timed steps include the landings on the plane
    torch.cuda.synchronize()
    # the timed steps are the NVTX range "sim_steps" (ncu --nvtx-include sim_steps/)
    torch.cuda.nvtx.range_push("sim_steps")
    t = time.perf_counter()
    st = ctx.sim_step(args.sim_steps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    torch.cuda.nvtx.range_pop()
    out = {"workload": SIM_WORKLOAD, "steps": args.sim_steps, "first_step": SIM_FIRST,
           "steps_per_s": args.sim_steps / dt,
           "newton_iterations_per_step": st["newton_iterations"] / args.sim_steps,
           "cg_iterations_per_newton": st["cg_iterations"] / max(st["newton_iterations"], 1)}
    # the same window with the line search's CCD on the piecewise-linear
    # trajectory (the reference's JSON default)
    ctx = rigc.Context(sc)
    ctx.sim_init(0.01, (0.0, -9.81, 0.0), 1e-3, trajectory="piecewise_linear")
    ctx.sim_step(SIM_FIRST)
    torch.cuda.synchronize()
    t = time.perf_counter()
    st = ctx.sim_step(args.sim_steps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    out["piecewise_linear"] = {"steps_per_s": args.sim_steps / dt,
                               "newton_iterations_per_step": st["newton_iterations"] / args.sim_steps}
    if not args.no_cpu_baseline:
        import oracle as O

        O.build()
        sim = O.OracleSim(sc, h=0.01, gravity=(0.0, -9.81, 0.0), dhat=1e-3)
        for _ in range(SIM_FIRST):
            sim.step()
        k, t = 0, time.perf_counter()
        while k < args.sim_steps and time.perf_counter() - t < 15.0:
            sim.step()
            k += 1
        out["cpu_oracle_steps_per_s"] = k / (time.perf_counter() - t)
    return out


def pass_rates(ctx, x0, x1, dhat, torch, reps=3):
    """ccd_pairs/s (continuous candidates x0 -> x1 through the CCD) and
    barrier_pairs/s (active constraints at x0 through energy, gradient, PSD
    12x12 Hessians, chain rule and BSR assembly), median of reps passes."""
    x0d, x1d = ctx.device(x0), ctx.device(x1)

    def timed(fn):
        ts = []
        for _ in range(reps + 1):
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t)
        return statistics.median(ts[1:])

    t_ccd = timed(lambda: ctx.compute_earliest_toi(x0d, x1d))
    s = ctx.stats()
    n_ccd = s["cand_ee"] + s["cand_fv"]
    cs = ctx.construct_constraint_set(x0d, dhat)
    n_con = len(cs["type"])
    t_bar = timed(lambda: (ctx.construct_constraint_set(x0d, dhat),
                           ctx.compute_barrier_term(x0d, dhat)))
    return {"ccd_candidates": n_ccd, "ccd_pairs_per_s": n_ccd / t_ccd, "ccd_ms": t_ccd * 1e3,
            "constraints": n_con, "barrier_pairs_per_s": n_con / t_bar, "barrier_ms": t_bar * 1e3}


def pass_rates_tuned(ctx, x0, x1, dhat, torch):
    """pass_rates with the built-in launch shapes, then after rigc_autotune
    on the same workload."""
    r = pass_rates(ctx, x0, x1, dhat, torch)
    tune = ctx.autotune(x0, x1, dhat)
    t = pass_rates(ctx, x0, x1, dhat, torch)
    r["tuned"] = {"ccd_pairs_per_s": t["ccd_pairs_per_s"],
                  "barrier_pairs_per_s": t["barrier_pairs_per_s"],
                  "choice": {k: tune[k] for k in ("ccd_blocks_per_sm", "cache_slots_per_body",
                                                  "ccd_seeds_log2", "ccd_hand_off", "ccd_warp",
                                                  "ccd_window_log2", "barrier_per_warp")}}
    return r


def settled(sc, steps, dhat, dt):
    """Poses after steps device time steps, and the explicit predictor from
    there (velocities of that state, gravity included) for the CCD pass."""
    import rigc

    c = rigc.Context(sc)
    c.sim_init(dt, (0.0, -9.81, 0.0), dhat)
    c.sim_step(steps)
    P, V, Q, _ = c.sim_state()
    x1 = P.copy()
    dyn = np.array([b.type == 2 for b in sc.bodies])
    x1[dyn, :3] += dt * V[dyn, :3]
    x1[dyn, 1] -= 9.81 * dt * dt
    return P.reshape(-1), x1.reshape(-1)


BARRIER_WORKLOAD = ("{n}x{n} columns of 2 tessellated slabs (1 x 0.2 x 1 m, faces of 32 x 32 "
                    "quads, 2,562 vertices each) resting 0.3 mm apart and on a static plane; "
                    "dhat 1e-3: constraint set, barrier energy, gradient, PSD-projected 12x12 "
                    "Hessians with the rigid chain rule, BSR assembly")


def barrier_rate(torch, n=4, reps=5):
    """The barrier terms at scale: the slab stacks' constraint set (some 10^5
    constraints), k_barrier_local alone (rigc_barrier_local_terms into device
    buffers, CUDA events on the context's stream) against its algorithmic
    bytes (1456 B per constraint), and the whole barrier pass (constraint set
    + compute_barrier_term with the BSR assembly)."""
    import rigc
    from rigc import scene as S

    sc = S.scene_from_json(S.spec_slab_stacks(0, nx=n, nz=n))
    ctx = rigc.Context(sc)
    dhat = sc.dhat
    x0 = sc.poses()
    xd = ctx.device(x0)
    cs = ctx.construct_constraint_set(xd, dhat)
    nc = len(cs["type"])
    dev = dict(dtype=torch.float64, device="cuda")
    e = torch.empty(nc, **dev)
    g = torch.empty((nc, 12), **dev)
    H = torch.empty((nc, 144), **dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ctx.barrier_local_terms_device(xd, nc, dhat, e, g, H)  # warm-up

    def timed(fn):
        ts = []
        for _ in range(reps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        return statistics.median(ts)

    t_local = timed(lambda: ctx.barrier_local_terms_device(xd, nc, dhat, e, g, H))
    t_pass = timed(lambda: (ctx.construct_constraint_set(xd, dhat),
                            ctx.compute_barrier_term(xd, dhat)))
    peak, kind = measured_peaks()
    achieved = BARRIER_BYTES_PER_CONSTRAINT * nc / t_local / 1e9
    types = np.bincount(np.asarray(cs["type"]), minlength=4)
    return {"workload": BARRIER_WORKLOAD.format(n=n), "bodies": sc.num_bodies,
            "constraints": nc,
            "constraint_types": {k: int(v) for k, v in zip(("vv", "ev", "ee", "fv"), types)},
            "k_barrier_local_ms": t_local * 1e3, "barrier_pass_ms": t_pass * 1e3,
            "barrier_constraints_per_s": nc / t_pass,
            "roofline": {"kernel": "k_body_frames + k_barrier_local", "bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": kind,
                         "bytes_per_constraint": BARRIER_BYTES_PER_CONSTRAINT}}


def per_config(args, torch):
    """Narrow-phase pass rates of the plain configurations beside the
    headline one: the 27-cube lattice and the 64-cube lattice after their
    landings (40 steps), and the 200-link chain (links 1.499 m apart, a 1 mm
    gap: at 1.5 they touch, see scene.spec_chain) once the links hang on each
    other (the constraint set at the current poses is not empty)."""
    import rigc
    from rigc import scene as S

    out = {}
    sc = S.scene_from_json(S.spec_cubes(args.seed))
    x0, x1 = settled(sc, 40, 1e-3, 0.01)
    out["cubes_27"] = pass_rates_tuned(rigc.Context(sc), x0, x1, 1e-3, torch)
    sc = S.scene_from_json(S.spec_cube_lattice(0))
    x0, x1 = settled(sc, 40, 1e-3, 0.01)
    out["cubes_64"] = pass_rates_tuned(rigc.Context(sc), x0, x1, 1e-3, torch)
    sc = S.scene_from_json(S.spec_chain(spacing=1.499))
    c = rigc.Context(sc)
    c.sim_init(0.005, (0.0, -9.81, 0.0), 1e-4)
    hanging = 0
    for _ in range(40):
        c.sim_step(5)
        hanging += 5
        P, _, _, _ = c.sim_state()
        if len(c.construct_constraint_set(P.reshape(-1), 1e-4)["type"]) > 0:
            break
    torch.cuda.synchronize()
    t = time.perf_counter()
    st = c.sim_step(5)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t
    P, V, Q, _ = c.sim_state()
    x1 = P.copy()
    dyn = np.array([b.type == 2 for b in sc.bodies])
    x1[dyn, :3] += 0.005 * V[dyn, :3]
    x1[dyn, 1] -= 9.81 * 0.005 ** 2
    r = pass_rates_tuned(rigc.Context(sc), P.reshape(-1), x1.reshape(-1), 1e-4, torch)
    r["steps_before"] = hanging
    r["steps_per_s"] = 5 / dt
    r["newton_iterations_per_step"] = st["newton_iterations"] / 5
    r["cg_iterations_per_newton"] = st["cg_iterations"] / max(1, st["newton_iterations"])
    out["chain_200"] = r
    return out


ADJOINT_WORKLOAD = ("64 unit cubes in a 4x4x4 lattice (spacing 1.05 m, seeded rotations, at rest) "
                    "landing on a static plane; 50 steps of 0.01 s, dhat 1e-3; loss |c0(T) - "
                    "(3, 0, 0.5)|^2; gradient over the 384 initial linear and angular velocities "
                    "by the device adjoint (checkpoints every 10 steps)")


def adjoint_rate(args, torch):
    """Forward rollout and adjoint of the differentiation workload through the
    torch.autograd.Function, and the oracle's rollout + adjoint on the host
    cores as its baseline."""
    from rigc import scene as S
    from rigc.adjoint import DIFF_DEFAULTS, DifferentiableSimulation, qdot_from_omega

    sc = S.scene_from_json(S.spec_cube_lattice(0))
    nb = sc.num_bodies
    steps = 50
    sim = DifferentiableSimulation(sc, 0.01, (0.0, -9.81, 0.0), 1e-3, checkpoint_every=10)
    dev = dict(dtype=torch.float64, device="cuda")
    poses = torch.as_tensor(sc.poses().reshape(nb, 6), **dev)
    vel = torch.as_tensor(sc.velocities().reshape(nb, 6), **dev)
    v = vel[:, :3].clone().requires_grad_()
    w = vel[:, 3:].clone().requires_grad_()
    target = torch.tensor([3.0, 0.0, 0.5], **dev)
    # warm-up: a short rollout and its backward (first-call set-up)
    Pw, _, _ = sim(poses, torch.cat([v, w], 1), qdot_from_omega(poses, w), 2)
    ((Pw[0, :3] - target) ** 2).sum().backward()
    v.grad = None
    w.grad = None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    P, _, _ = sim(poses, torch.cat([v, w], 1), qdot_from_omega(poses, w), steps)
    loss = ((P[0, :3] - target) ** 2).sum()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    loss.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    out = {"workload": ADJOINT_WORKLOAD, "parameters": 6 * (nb - 1), "steps": steps,
           "forward_s": t1 - t0, "backward_s": t2 - t1, "gradients_per_s": 1.0 / (t2 - t0),
           "newton_iterations": sim.stats["newton_iterations"], "loss": float(loss.detach())}
    if not args.no_cpu_baseline:
        import oracle as O

        O.build()
        osim = O.OracleSim(sc, h=0.01, gravity=(0.0, -9.81, 0.0), dhat=1e-3,
                           **{k: int(v) if isinstance(v, bool) else v
                              for k, v in DIFF_DEFAULTS.items()})
        t = time.perf_counter()
        osim.rollout(steps, record=True)
        dp = np.zeros((nb, 6))
        dp[0, :3] = 2 * (osim.pose.reshape(nb, 6)[0, :3] - np.array([3.0, 0.0, 0.5]))
        osim.backward(dp)
        out["cpu_oracle_s"] = time.perf_counter() - t
        out["cpu_oracle_cores"] = os.cpu_count()
    return out


BATCH_WORKLOAD = ("{n} scenes, each a seeded count U[8, 512] of convex hulls of 32 random "
                  "unit-sphere points (scale U[0.5, 2.0]) in a contact pile (2e-4 m gaps) on its "
                  "own static plane; dhat 1e-3; one narrow-phase pass per scene")


def _hull_scene(seed):
    """One scene of the batched form with its pile poses and predictor poses."""
    from rigc import scene as S

    rng = np.random.default_rng(seed)
    n = int(rng.integers(8, 513))
    sc = S.scene_from_json(S.spec_hulls(seed, n))
    x0 = S.packed_pile_poses(sc, seed=seed)
    return sc, x0, sc.predictor_poses(x0)


def batched_rate(args, torch):
    """Candidate pairs per second of one narrow-phase pass over many small
    scenes: one batched context (all scenes in the same launches) against one
    context per scene run one after the other (the plain path)."""
    import multiprocessing as mp

    import rigc
    from rigc import scene as S

    seeds = [10_000 + args.seed * 1000 + k for k in range(args.batch_scenes)]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        items = pool.map(_hull_scene, seeds)
    scenes = [sc for sc, _, _ in items]
    big, sob = S.concat_scenes(scenes)
    X0 = np.concatenate([x for _, x, _ in items])
    X1 = np.concatenate([x for _, _, x in items])
    dhat = scenes[0].dhat

    def run_pass(ctx, x0, x1):
        ctx.compute_earliest_toi(x0, x1)
        s = ctx.stats()
        ctx.construct_constraint_set(x0, dhat)
        ctx.compute_barrier_term(x0, dhat)
        s2 = ctx.stats()
        return s["cand_ee"] + s["cand_fv"] + s2["cand_ee"] + s2["cand_fv"]

    cb = rigc.Context(big, scene_of_body=sob)
    x0d, x1d = cb.device(X0), cb.device(X1)

    def timed_passes():
        for _ in range(2):
            run_pass(cb, x0d, x1d)
        torch.cuda.synchronize()
        t = time.perf_counter()
        pairs = 0
        reps = 3
        for _ in range(reps):
            pairs += run_pass(cb, x0d, x1d)
        torch.cuda.synchronize()
        return pairs // reps, (time.perf_counter() - t) / reps

    pairs_untuned, t_untuned = timed_passes()
    # launch shapes chosen by the autotuner on this batch
    tune = cb.autotune(x0d, x1d, dhat)
    pairs_b, tb = timed_passes()
    ctxs = [(rigc.Context(sc), None) for sc in scenes]
    dev = [(c.device(x0), c.device(x1)) for (c, _), (_, x0, x1) in zip(ctxs, items)]
    for (c, _), (a, b) in zip(ctxs, dev):
        run_pass(c, a, b)
    torch.cuda.synchronize()
    t = time.perf_counter()
    pairs_p = 0
    for (c, _), (a, b) in zip(ctxs, dev):
        pairs_p += run_pass(c, a, b)
    torch.cuda.synchronize()
    tp = time.perf_counter() - t
    out = {"workload": BATCH_WORKLOAD.format(n=args.batch_scenes), "bodies": big.num_bodies,
           "pairs_per_pass": pairs_b, "batched_pairs_per_s": pairs_b / tb,
           "plain_pairs_per_s": pairs_p / tp, "batched_ms": tb * 1e3, "plain_ms": tp * 1e3,
           "batched_untuned_ms": t_untuned * 1e3, "autotune": tune}
    del ctxs, dev, cb
    if args.batch_sim_steps > 0:
        out["sim"] = batched_sim_rate(args, torch, items, big, sob, tune)
    return out


def batched_sim_rate(args, torch, items, big, sob, tune):
    """Simulated scene-steps per second: every scene from its contact pile
    with its seeded velocities, one time step (the full IPC Newton solve) per
    scene per step -- one batched context stepping all scenes at once
    against one context per scene on a fixed sample of the scenes."""
    import rigc

    scenes = [sc for sc, _, _ in items]
    X0 = np.concatenate([x for _, x, _ in items]).reshape(-1, 6)
    dhat = scenes[0].dhat
    grav = (0.0, -9.81, 0.0)
    K = args.batch_sim_steps
    cb = rigc.Context(big, scene_of_body=sob)
    cb.set_tune(tune["ccd_blocks_per_sm"], tune["cache_slots_per_body"], tune["barrier_per_warp"],
                tune["ccd_seeds_log2"], tune["ccd_hand_off"], tune["ccd_warp"])
    cb.set_ccd_window(tune["ccd_window_log2"])
    cb.sim_init(0.01, grav, dhat, poses=X0)
    cb.sim_step(1)
    torch.cuda.synchronize()
    t = time.perf_counter()
    st = cb.sim_step(K)
    torch.cuda.synchronize()
    tb = time.perf_counter() - t
    sample = list(range(0, len(scenes), max(1, len(scenes) // args.batch_sim_plain_sample)))
    tp, its = 0.0, 0
    for k in sample:
        sc, x0, _ = items[k]
        c = rigc.Context(sc)
        c.sim_init(0.01, grav, dhat, poses=x0)
        c.sim_step(1)
        torch.cuda.synchronize()
        t = time.perf_counter()
        sp = c.sim_step(K)
        torch.cuda.synchronize()
        tp += time.perf_counter() - t
        its += sp["newton_iterations"]
        del c
    sb = sum(scenes[k].num_bodies for k in sample)
    return {"steps": K, "scenes": len(scenes), "batched_scene_steps_per_s": len(scenes) * K / tb,
            "batched_s_per_step": tb / K,
            "batched_newton_iterations_per_scene_step": st["newton_iterations"] / (len(scenes) * K),
            "plain_scene_steps_per_s": len(sample) * K / tp,
            "plain_sample": f"{len(sample)} of the scenes ({sb} bodies), one context each",
            "plain_newton_iterations_per_scene_step": its / (len(sample) * K)}


def run_reference(args):
    """The CPU path of the reference restated (oracle) on the machine's cores:
    each step one whole narrow-phase pass of the workload, timed."""
    if args.gpus > 1 and int(os.environ.get("RANK", "0")) != 0:
        return
    sc, x0, x1 = make_workload(args.bodies, args.seed)
    import oracle as O

    O.build()
    o = O.OracleScene(sc)
    dhat = sc.dhat
    nthreads = os.cpu_count() or 1
    ee, fv = o.detect_candidates(x0, x1, True, 0.0)
    ee_d, fv_d = o.detect_candidates(x0, continuous=False, inflation=dhat / 2)
    n_ccd, n_disc = len(ee) + len(fv), len(ee_d) + len(fv_d)
    times = []
    for s in range(args.warmup + args.steps):
        dt = cpu_pass(o, x0, x1, dhat, nthreads)
        if s >= args.warmup:
            times.append(dt)
    total = sum(times)
    v = (n_ccd + n_disc) * len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / len(times) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.bodies} icospheres (subdivision 3) contact pile, one "
                               "narrow-phase pass", "ccd_candidates": n_ccd,
                   "discrete_candidates": n_disc},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": CPU_SAMPLE.format(n=nthreads)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    import torch

    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    import rigc

    sc, x0, x1 = make_workload(args.bodies, args.seed + rank)
    dhat = sc.dhat
    ctx = rigc.Context(sc)
    x0d, x1d = ctx.device(x0), ctx.device(x1)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        toi = ctx.compute_earliest_toi(x0d, x1d)
        ctx.construct_constraint_set(x0d, dhat)
        e, g, H = ctx.compute_barrier_term(x0d, dhat)
        return toi

    # sizes
    ee, fv = ctx.detect_collision_candidates_rigid(x0d, x1d, True, 0.0)
    n_ccd = len(ee) + len(fv)
    ee_d, fv_d = ctx.detect_collision_candidates_rigid(x0d, x0d, False, dhat / 2)
    n_disc = len(ee_d) + len(fv_d)
    cs = ctx.construct_constraint_set(x0d, dhat)
    n_cons = len(cs["type"])
    # launch shapes chosen by the autotuner on this workload (part of the
    # framework's set-up, before the warm-up)
    tune = None
    if args.ccd_warp is not None:
        ctx.set_tune(0, 0, 0, -1, -1, args.ccd_warp)
        tune = {"ccd_warp": args.ccd_warp, "forced": True}
    elif not args.no_autotune:
        tune = ctx.autotune(x0d, x1d, dhat)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = ctx.stats()["kernel_launches"]
    times = []
    with ClockSampler() as clk:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            step()
            b.record()
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b) / 1e3)
        if world > 1:
            torch.distributed.barrier()
    launches = ctx.stats()["kernel_launches"] - launches0
    total = sum(times)
    if world > 1:
        t = torch.tensor([total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total = float(t.item())
    ms = total / args.steps * 1e3
    value = world * (n_ccd + n_disc) * args.steps / total

    # per-phase timing (kernel-level, resident inputs, after an L2 flush)
    def timed(fn, reps=3):
        best = []
        for _ in range(reps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            best.append(a.elapsed_time(b) / 1e3)
        return statistics.median(best)

    # one untimed compute_earliest_toi in the NVTX range "ccd_call": its
    # CCD launches (ncu --nvtx-include ccd_call/ -k regex:k_ccd) give the
    # DRAM traffic of one CCD call as the step makes it
    torch.cuda.nvtx.range_push("ccd_call")
    ctx.compute_earliest_toi(x0d, x1d)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    st = ctx.stats()
    # one untimed continuous broad phase in the NVTX range "bp_call"
    torch.cuda.nvtx.range_push("bp_call")
    ctx.count_collision_candidates_rigid(x0d, x1d, True, 0.0)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    # the broad phase with the candidates left on the device, and the CCD as
    # the step runs it: compute_earliest_toi (broad phase, then the CCD taking
    # over its frames) less the broad phase
    t_bp = timed(lambda: ctx.count_collision_candidates_rigid(x0d, x1d, True, 0.0))
    t_ccd = timed(lambda: ctx.compute_earliest_toi(x0d, x1d)) - t_bp
    ctx.construct_constraint_set(x0d, dhat)
    t_bar = timed(lambda: ctx.compute_barrier_term(x0d, dhat))

    # end to end from host buffers
    e2e_times = []
    nb = sc.num_bodies
    for i in range(args.warmup + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t = time.perf_counter()
        toi, energy, grad, (rp, col, val), nnzb = ctx.narrow_phase_host(x0, x1, dhat)
        t = time.perf_counter() - t
        if i >= args.warmup:
            e2e_times.append(t)
    e2e = (n_ccd + n_disc) / statistics.median(e2e_times)
    h2d = 2 * 6 * nb * 8
    d2h = 6 * nb * 8 + (nb + 1) * 4 + nnzb * (4 + 36 * 8)

    peak, peak_kind = measured_peaks()
    # the CCD kernel the context launches: one search per warp unless tuned
    # otherwise
    ccd_mode = tune.get("ccd_warp", -1) if tune else -1
    ccd_kernel = CCD_KERNELS.get(ccd_mode, "k_ccd_group<32, 1>")
    fp64 = fp64_peak() if rank == 0 else None
    ccd_bytes = CCD_BYTES_PER_PAIR * n_ccd
    achieved = ccd_bytes / t_ccd / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.bodies} icospheres (subdivision 3) contact pile, one "
                               "narrow-phase pass (CCD broad+narrow, constraint set, "
                               "barrier grad + PSD Hessian, BSR assembly)",
                   "ccd_candidates": n_ccd, "discrete_candidates": n_disc,
                   "constraints": n_cons, "ccd_boxes": st["ccd_boxes"],
                   "ccd_collisions": st["ccd_collisions"], "l2": "flushed (512 MiB write) "
                   "before every timed step", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "phases_s": {"ccd_narrow": t_ccd, "ccd_broad": t_bp, "barrier_and_assembly": t_bar},
        "broad_phase_roofline": broad_phase_roofline(sc, n_ccd, t_bp, peak, peak_kind),
        "ccd_pairs_per_s": n_ccd / t_ccd, "barrier_constraints_per_s": n_cons / t_bar,
        "roofline": {"bound": "hbm", "kernel": ccd_kernel, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (K_CCD_DRAM_BYTES_PER_CANDIDATE[ccd_kernel] * n_ccd
                                 if ccd_kernel in K_CCD_DRAM_BYTES_PER_CANDIDATE else None),
                     "traffic_source": "ncu capture of the 200-icosphere pile scaled by candidates",
                     "peak_source": peak_kind,
                     "note": "FP64-issue-bound (an FP64 warp instruction holds its SM "
                             "sub-partition's FP64 unit 64 cycles on GB300), not HBM: algorithmic "
                             "bytes are 304 B per candidate",
                     "fp64": fp64_roofline(K_CCD_FP64.get(ccd_kernel), fp64)},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "clocks": clk.summary(),
        "fp64_peak": fp64,
        "gpu_launches": launches,
        "autotune": tune,
    }
    if rank == 0 and not args.no_sim:
        line["steps_per_s"] = sim_rate(args, torch)
    if rank == 0 and args.batch_scenes > 0:
        line["batched"] = batched_rate(args, torch)
    if rank == 0 and not args.no_adjoint:
        line["adjoint"] = adjoint_rate(args, torch)
    if rank == 0 and not args.no_configs:
        line["per_config"] = per_config(args, torch)
    if rank == 0 and not args.no_barrier:
        line["barrier_at_scale"] = barrier_rate(torch, n=args.barrier_columns)
    if rank == 0 and not args.no_pl:
        line["piecewise_linear"] = pl_rate(ctx, sc, x0, x1, x0d, x1d, timed,
                                           with_cpu=not args.no_cpu_baseline)
    if rank == 0 and not args.no_cpu_baseline:
        base = cpu_baseline(sc, x0, x1, dhat)
        line["cpu_baseline"] = {"value": base["pairs_per_s"], "unit": UNIT, "cores": base["cores"],
                                "kind": "port", "sample": base["sample"],
                                "pass_ms": base["pass_s"] * 1e3}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
