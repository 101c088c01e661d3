#!/usr/bin/env python3
"""Benchmark of the ICEP per-timestep hot path on GB300.

Workload (one "step" = one Time_evolution_hydro step, Electrolyte +
Dielectric_property ON): periodic 128^3 grid, dx = 1; 512 rigid spheres a = 4,
xi = 2 (volume fraction 6.5%) at seeded random positions with minimum
separation 10; per-particle permittivity uniform in [1, 5] (seeded),
eps_fluid = 80; uniform field E0 = (0, 0, 0.1); salt z = +-1, Onsager 7.24,
Debye length 10 a, kBT = 1; dt = 0.01; Poisson solved to 1e-8 relative true
residual: float-float iterative refinement around the plain spectral-
preconditioned inner solve (CG; BiCGSTAB with ICEP_INNER=bicgstab). Synthetic
inputs only (no dataset is involved).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0). --impl reference runs the CPU restatement of
the reference's own algorithm (oracle/, FP64, all host threads) on the same
workload: one full step of it takes longer than a benchmark run allows, so it
prints an `unavailable` line with the one step it timed.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "ICEP steps/s at 128^3, learned-precond vs plain on GB300 at 1e-8 residual; HBM %"
UNIT = "steps/s"

# Dominant kernel of the step (largest share of device time in the ncu launch
# list of this bench, profiles/launches_icep_step_128.txt) and its probe id.
PROBE_KERNEL = "k_kop_plane_r<128,64> (fused plane pass of the k-space Poisson operator, 3 components)"
PROBE_KIND = 1
# DRAM bytes (read + write) per launch of that kernel from one ncu capture
# (profiles/k_kop_plane_128.txt), keyed by (grid, precision, kernel).
TRAFFIC = {(128, "mixed", PROBE_KERNEL): 42.90e6}


def workload(args, precision, solver):
    import cases
    from icep_kapsel_gb300 import abi
    p, parts = cases.icep_case(n=args.n, npart=args.np, minsep=10.0, seed=2024, a=4.0, eps_f=80.0, eps_p=3.0,
                               e_ext=(0.0, 0.0, 0.1), tol=args.tol, maxit=args.maxit, dt=0.01,
                               per_particle_eps=(1.0, 5.0), solver=solver, precision=precision)
    return p, parts


def solver_label(precision):
    from icep_kapsel_gb300 import abi
    if precision == abi.FP64:
        return "spectral-preconditioned BiCGSTAB, FP64 (plain)"
    inner = "BiCGSTAB" if os.environ.get("ICEP_INNER") == "bicgstab" else "CG"
    return "spectral-preconditioned %s inner solve, float-float true-residual refinement (plain)" % inner


def workload_config(args, precision_name, solver_name):
    return {"workload": "icep_step_%d^3_%d_spheres" % (args.n, args.np), "grid": [args.n] * 3,
            "particles": args.np, "radius": 4.0, "xi": 2.0, "eps_fluid": 80.0,
            "eps_particle": "uniform[1,5] per particle", "E0": [0.0, 0.0, 0.1], "poisson_tol": args.tol,
            "poisson_solver": solver_name, "precision": precision_name, "dt": 0.01,
            "l2_policy": "working set larger than L2 (every step touches ~40 grid fields)",
            "seed": 2024}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for ln in open(self.path):
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # one replica per GPU: make this rank's GPU the only visible one
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, local, None


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


base_oracle = [None]


def mixed_error(args, o, nsteps):
    """Per-field relative L2 error of the MIXED GPU path against the FP64
    oracle after the same `nsteps` steps of the workload (same algorithm:
    spectral-preconditioned solve to the same true residual)."""
    import cases
    from icep_kapsel_gb300 import abi
    from icep_kapsel_gb300.runtime import Simulation
    p, parts = workload(args, abi.MIXED, abi.SOLVER_SPECTRAL)
    m = Simulation(p, parts)
    m.init_state()
    m.step(nsteps)
    e = cases.mixed_vs_oracle_errors(m, o, args.n, args.np)
    m.close()
    return {"steps": nsteps, "relative_l2": e,
            "fields": "zeta0/zeta1 vorticity, u velocity, phi profile, pot potential (mean removed), "
                      "c0/c1 ion densities, particle_x/particle_v positions/velocities"}


def cpu_baseline(args, sample_steps=8):
    """The oracle (FP64 C restatement, all host threads) on a bounded sample of
    the same workload, with the GPU path's algorithm (spectral-preconditioned
    Poisson solve): `sample_steps` full steps after one warm-up step."""
    import pyoracle
    from icep_kapsel_gb300 import abi
    p, parts = workload(args, abi.FP64, abi.SOLVER_SPECTRAL)
    o = pyoracle.Oracle(p, parts)
    o.init_state()
    o.step(1)
    it = []
    t0 = time.perf_counter()
    for _ in range(sample_steps):
        o.step(1)
        it.append(o.last_iterations())
    dt = time.perf_counter() - t0
    cores = o.lib.ko_max_threads()
    base_oracle[0] = o  # its state after 1 + sample_steps steps, for the MIXED error
    return {"value": sample_steps / dt, "unit": UNIT, "cores": int(cores), "kind": "port",
            "sample": "%d full steps (after 1 warm-up step) of the %d^3 / %d-sphere workload: FP64 C restatement, "
                      "OpenMP, spectral-preconditioned Poisson solve to %g (%s iterations per step), %.1f s"
                      % (sample_steps, args.n, args.np, args.tol, "/".join(map(str, it)), dt)}


def run_reference(args, world, rank, dist):
    """CPU reference arm: the reference's algorithm (the oracle's restatement
    of Charge_field2potential_dielectric_LO, operate_dielectric.cxx:542-572:
    identity-preconditioned BiCGSTAB with the MaxIter retry from a zero guess,
    FP64, all host threads) on the same workload.

    A full step of it does not fit into a benchmark run: on this workload the
    solve needs ~150 iterations (~300 operator applications of 8 FFTs each)
    per step for the first steps, and from the sixth step on both MaxIter
    attempts stagnate above the 1e-8 tolerance (~4000 operator applications,
    minutes per step). So the arm prints its `unavailable` line with that
    reason and, in a separate field, the one real full step it did time: the
    initial solve and the first step of the workload, each a complete
    reference solve to 1e-8, with their operator-application counts."""
    if rank != 0:
        return
    import pyoracle
    from icep_kapsel_gb300 import abi
    p, parts = workload(args, abi.FP64, abi.SOLVER_REF)
    o = pyoracle.Oracle(p, parts)
    cores = int(o.lib.ko_max_threads())
    t0 = time.perf_counter()
    o.init_state()
    t_init = time.perf_counter() - t0
    m_init, it_init, err_init = o.matvecs(), o.last_iterations(), o.last_error()
    t0 = time.perf_counter()
    o.step(1)
    t_step = time.perf_counter() - t0
    m_step, it_step, err_step = o.matvecs() - m_init, o.last_iterations(), o.last_error()
    # from the sixth step on the solve stagnates above the tolerance and runs
    # both MaxIter attempts: 2 * (MaxIter + 1) operator applications
    t_stagnant = t_step * 2.0 * (args.maxit + 1) / max(m_step, 1)
    need_min = (min(args.steps + args.warmup, 5) * t_step + max(args.steps + args.warmup - 5, 0) * t_stagnant) / 60.0
    line = {"impl": "reference", "metric": METRIC, "unit": UNIT, "higher_is_better": True, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "unavailable": ("a full reference step of the %d^3 / %d-sphere workload took %.1f s on %d host cores "
                            "(%d operator applications); from the sixth step on its solve stagnates above the "
                            "tolerance and runs both MaxIter attempts (~%.0f s a step at the same rate), so "
                            "--steps %d --warmup %d would take about %.0f min"
                            % (args.n, args.np, t_step, cores, m_step, t_stagnant, args.steps, args.warmup,
                               need_min)),
            "config": workload_config(args, "fp64", "reference BiCGSTAB (identity)"),
            "one_full_step": {"seconds": t_step, "steps_per_s": 1.0 / t_step, "cores": cores, "kind": "port",
                              "iterations": int(it_step), "operator_applications": int(m_step),
                              "relative_residual": err_step,
                              "initial_solve": {"seconds": t_init, "iterations": int(it_init),
                                                "operator_applications": int(m_init),
                                                "relative_residual": err_init},
                              "sample": "the initial Poisson solve and the first step of the workload, timed "
                                        "once each (a real full step, not a projection)"}}
    print(json.dumps(line), flush=True)


def run_gpu(args, world, rank, local, dist):
    from icep_kapsel_gb300 import abi
    from icep_kapsel_gb300.build import build
    build()
    from icep_kapsel_gb300.runtime import Simulation, load_library
    lib = load_library()
    lib.icep_step_timed.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    lib.icep_kernel_launches.restype = C.c_ulonglong
    lib.icep_algorithmic_bytes.restype = C.c_ulonglong
    lib.icep_probe_start.argtypes = [C.c_int, C.c_int]
    lib.icep_probe_stop.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.POINTER(C.c_double)]
    lib.icep_pin_host.argtypes = [C.c_void_p, C.c_size_t]
    lib.icep_unpin_host.argtypes = [C.c_void_p]
    precision = abi.MIXED if args.precision == "mixed" else abi.FP64
    p, parts = workload(args, precision, abi.SOLVER_SPECTRAL)
    sim = Simulation(p, parts)
    tiles = None
    if precision == abi.MIXED:
        picks, us = sim.autotune_picks()
        tiles = {"xinv_pencils_per_block": picks[0], "xfwd_pencils_per_block": picks[1],
                 "plane_kernel": "shared-memory" if picks[2] else "register-resident",
                 "us_per_launch": {"xinv_8_16_32": list(us[0:3]), "xfwd_8_16_32": list(us[3:6]),
                                   "plane_register_shared": list(us[6:8])}}
    sim.init_state()
    for _ in range(args.warmup):
        sim.step(1)
    sim.synchronize()
    if dist is not None:
        dist.barrier()
    ms = C.c_double(0)
    launches0 = lib.icep_kernel_launches()
    abytes0 = lib.icep_algorithmic_bytes()
    graphs0 = sim.step_graphs()
    with ClockSampler(0) as clk:
        st = lib.icep_step_timed(sim.ctx, args.steps, C.byref(ms))
    if st != 0:
        raise RuntimeError("timed steps failed: %d" % st)
    launches = int(lib.icep_kernel_launches() - launches0)
    graph_steps = sim.step_graphs() - graphs0
    step_bytes = float(lib.icep_algorithmic_bytes() - abytes0) / args.steps
    # the dominant kernel's launches timed with CUDA events on their stream
    # over further steps (the probe's events run the solver's iterations as
    # plain launches, not replayed graphs; the kernel itself is the same)
    probe_steps = min(args.steps, 5)
    lib.icep_probe_start(PROBE_KIND, 1 << 16)
    pstat = lib.icep_step_timed(sim.ctx, probe_steps, C.byref(C.c_double(0)))
    pms, pn, pbytes = C.c_double(0), C.c_longlong(0), C.c_double(0)
    lib.icep_probe_stop(C.byref(pms), C.byref(pn), C.byref(pbytes))
    if pstat != 0:
        raise RuntimeError("probe steps failed: %d" % pstat)
    iters, err, _ = sim.solver_stats()
    t_ms = reduce_max(dist, ms.value)
    if dist is not None:
        dist.barrier()
    value = world * args.steps / (t_ms / 1000.0)
    peak, peak_kind = measured_peaks()
    step_gbs = step_bytes / (t_ms / args.steps * 1e-3) / 1e9
    achieved = pbytes.value / (pms.value * 1e-3) / 1e9 if pms.value > 0 else None
    per_launch_bytes = pbytes.value / pn.value if pn.value else None
    traffic = TRAFFIC.get((args.n, args.precision, PROBE_KERNEL))

    # end to end: the drop-in Time_evolution call on pinned host arrays
    shp = (p.nx, p.ny, 2 * (p.nz // 2 + 1))
    host = {k: np.ascontiguousarray(sim.get(k)) for k in ("zeta0", "zeta1", "c0", "c1", "pot")}
    ukdc = np.ascontiguousarray(sim.uk_dc())
    hparts = sim.particles()
    for a in host.values():
        lib.icep_pin_host(a.ctypes.data, a.nbytes)
    lib.icep_pin_host(C.addressof(hparts), C.sizeof(hparts))
    field_bytes = int(np.prod(shp)) * 8
    io_bytes = 5 * field_bytes + 3 * 8 + C.sizeof(hparts)
    sim.time_evolution(host["zeta0"], host["zeta1"], ukdc, hparts, host["c0"], host["c1"], host["pot"], 1)
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.time_evolution(host["zeta0"], host["zeta1"], ukdc, hparts, host["c0"], host["c1"], host["pot"], 1)
    e2e_s = reduce_max(dist, time.perf_counter() - t0)
    for a in host.values():
        lib.icep_unpin_host(a.ctypes.data)
    lib.icep_unpin_host(C.addressof(hparts))
    e2e = world * args.steps / e2e_s
    sim.close()
    learned = None if (args.no_learned or args.precision != "mixed") else run_learned(args, lib, value)
    batched = None if (args.no_batch or args.precision != "mixed") else run_batch(args)
    large = None if (args.no_large or args.precision != "mixed" or world > 1) else run_large(args, lib)
    if rank != 0:
        return
    base = None
    fp64_error = None
    if not args.no_cpu_baseline:
        base = cpu_baseline(args)
        if args.precision == "mixed":
            fp64_error = mixed_error(args, base_oracle[0], 9)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if precision == abi.FP64 else "f32 (fields, FFTs, inner Krylov) + f64 (particles, k=0, residual)",
            "data": "synthetic",
            "config": dict(workload_config(args, args.precision, solver_label(precision)),
                           parallelism="replicas" if world > 1 else "single GPU"),
            "poisson": {"iterations_last_solve": iters, "relative_true_residual": err},
            "clocks": clk.summary(),
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes},
            "gpu_launches": launches,
            # the timed launches' positions in the process's launch sequence
            # (for slicing a profiler's launch list to the timed steps)
            "timed_launch_range": [int(launches0), int(launches0) + launches],
            "steps_as_one_graph": graph_steps,
            "grid_point_steps_per_s": value * args.n ** 3,
            "roofline": {"bound": "hbm", "kernel": PROBE_KERNEL, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind + " (hbm_gbs, copy)", "unit": "GB/s",
                         "frac": achieved / peak if achieved else None, "traffic": traffic,
                         "launches_timed": pn.value, "ms_per_launch": pms.value / pn.value if pn.value else None,
                         "bytes_per_launch": per_launch_bytes,
                         "step": {"algorithmic_bytes_per_step": step_bytes, "achieved": step_gbs, "peak": peak,
                                  "unit": "GB/s", "frac": step_gbs / peak,
                                  "definition": "every kernel of the step adds its external inputs and outputs "
                                                "(icep_algorithmic_bytes), summed over the timed steps, divided "
                                                "by the steps' device time"}},
            "cpu_baseline": base, "autotune": tiles}
    if fp64_error is not None:
        line["fp64_oracle_error"] = fp64_error
    if learned is not None:
        line["learned"] = learned
    if batched is not None:
        line["batched"] = batched
    if large is not None:
        line["large"] = large
    print(json.dumps(line), flush=True)


def run_batch(args, n_replicas=64, seed=4242):
    """The batched ensemble: independent replicas with meshes drawn from
    {32^3, 64^3} (the path supports power-of-two meshes, as the reference),
    8-16 spheres at 32^3 and 8-64 at 64^3 (a = 4, xi = 2, seeded positions,
    eps_p uniform in [1, 5]), |E0| uniform in [0.05, 0.2], advanced together
    by icep_batch_step. Value: replica-steps per second over the batch."""
    import cases
    from icep_kapsel_gb300 import abi
    from icep_kapsel_gb300.runtime import Batch
    rng = np.random.default_rng(seed)
    reps, points = [], 0
    for i in range(n_replicas):
        n = int(rng.choice([32, 64]))
        npart = int(rng.integers(8, 17 if n == 32 else 65))
        ez = float(rng.uniform(0.05, 0.2))
        reps.append(cases.icep_case(n=n, npart=npart, minsep=10.0, seed=seed + i, a=4.0, eps_f=80.0, eps_p=3.0,
                                    e_ext=(0.0, 0.0, ez), tol=args.tol, maxit=args.maxit, dt=0.01,
                                    per_particle_eps=(1.0, 5.0), solver=abi.SOLVER_SPECTRAL,
                                    precision=abi.MIXED))
        points += n ** 3
    b = Batch(reps)
    lib = b.lib
    lib.icep_kernel_launches.restype = C.c_ulonglong
    b.init_state()
    b.step(args.warmup)
    g0 = [b.replica(i).step_graphs() for i in range(n_replicas)]
    l0 = lib.icep_kernel_launches()
    t0 = time.perf_counter()
    b.step(args.steps)
    dt = time.perf_counter() - t0
    l1 = lib.icep_kernel_launches()
    # batch steps taken as one graph launch: every replica's step replayed
    graph_steps = min(b.replica(i).step_graphs() - g0[i] for i in range(n_replicas))
    b.close()
    return {"replicas": n_replicas, "meshes": "32^3 / 64^3", "value": n_replicas * args.steps / dt,
            "unit": "replica-steps/s", "grid_point_steps_per_s": points * args.steps / dt,
            "ms_per_batch_step": 1000.0 * dt / args.steps,
            "batch_steps_as_one_graph_launch": graph_steps,
            "kernel_launches_per_batch_step": (l1 - l0) / args.steps,
            "timing": "host wall clock around icep_batch_step (returns after every replica has finished)"}


def dense_positions(n, L, minsep, seed, max_tries=2000000):
    """n centres uniform in [0, L)^3 with periodic separation >= minsep
    (random sequential addition, vectorised over the accepted centres)."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 3))
    k = tries = 0
    while k < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("cannot place %d spheres with separation %g" % (n, minsep))
        x = rng.uniform(0.0, L, 3)
        if k:
            d = out[:k] - x
            d -= L * np.round(d / L)
            if np.min(np.einsum("ij,ij->i", d, d)) < minsep * minsep:
                continue
        out[k] = x
        k += 1
    return out


def run_large(args, lib, n=256, npart=2048, a=7.3, seed=2561):
    """One 256^3 system with 2048 dielectric spheres at volume fraction 0.2
    (a = 7.3, xi = 2, centres at least 16.6 apart so that no pair starts
    inside the Lennard-Jones cutoff; eps_p uniform in [1, 5], eps_f = 80,
    E0 = (0, 0, 0.1), Poisson to 1e-8), MIXED precision: steps/s and
    grid-point-steps/s of the timed steps (CUDA events)."""
    from icep_kapsel_gb300 import abi
    from icep_kapsel_gb300.runtime import Simulation
    x = dense_positions(npart, float(n), 2 * a + 2.0, seed)
    eps = np.random.default_rng(seed + 1).uniform(1.0, 5.0, npart)
    p = abi.make_params(nx=n, ny=n, nz=n, n_particles=npart, n_species=1, sw_eq=abi.ELECTROLYTE, dielectric=1,
                        dielectric_cst=1.0, eps_fluid=80.0, eps_particle_top=3.0, eps_particle_bottom=3.0,
                        external_field=1, e_ext=[0.0, 0.0, 0.1], potential_tol=args.tol, potential_iter=args.maxit,
                        kbt=1.0, debye_length=10.0, onsager_pos=7.24, onsager_neg=7.24, valency_pos=1.0,
                        valency_neg=-1.0, dt=0.01, a=a, a_xi=2.0, rotation=0, per_particle_eps=1,
                        solver=abi.SOLVER_SPECTRAL, precision=abi.MIXED)
    sim = Simulation(p, abi.make_particles(x, eps_p=eps))
    sim.init_state()
    for _ in range(2):
        sim.step(1)
    ms = C.c_double(0)
    k = 4
    if lib.icep_step_timed(sim.ctx, k, C.byref(ms)) != 0:
        raise RuntimeError("256^3 timed steps failed")
    it, err, _ = sim.solver_stats()
    sim.close()
    v = k / (ms.value / 1000.0)
    vf = npart * 4.0 / 3.0 * np.pi * a ** 3 / float(n) ** 3
    return {"workload": "icep_step_%d^3_%d_spheres_vf%.2f" % (n, npart, vf), "value": v, "unit": UNIT,
            "ms_per_step": ms.value / k, "grid_point_steps_per_s": v * n ** 3, "steps": k, "warmup": 2,
            "poisson": {"iterations_last_solve": it, "relative_true_residual": err}}


def run_learned(args, lib, plain_value):
    """The same workload with the learned preconditioner (solver LEARNED):
    the network is trained on the GPU first (outside the timed region), then
    K steps are timed as for the plain solver; also timed with the network
    switched off (flexible GMRES with the spectral preconditioner only)."""
    from icep_kapsel_gb300 import abi
    from icep_kapsel_gb300.runtime import Simulation
    p, parts = workload(args, abi.MIXED, abi.SOLVER_LEARNED)
    sim = Simulation(p, parts)
    sim.init_state()
    # held-out residuals: the workload's own right-hand side and the next
    # residuals of its spectral iteration (no training configuration is it)
    sim.learned_enable(1)
    ls0, ll0 = sim.learned_eval(4)  # the network with its initial weights
    sim.learned_enable(0)
    configs, steps = 200, 20
    t0 = time.perf_counter()
    l0, l1 = sim.learned_train(configs=configs, steps=steps, seed=3, lr=1e-3)
    sim.synchronize()
    t_train = time.perf_counter() - t0
    ls, ll = sim.learned_eval(4)  # the network counts only if training was kept
    out = {"train": {"adam_steps": configs * steps, "configurations": configs,
                     "particles_per_configuration": "%d..%d present, eps_p uniform in [1, 10]" % (args.np // 4, args.np),
                     "seconds": t_train, "loss_first_step": l0, "loss_last_step": l1},
           "held_out_one_step_loss": {"spectral_only": ls, "network_initial_weights": ll0, "network_trained": ll,
                                      "gain_vs_spectral": 1.0 - ll / ls, "training_kept": bool(ll < ls)}}
    for key, on in (("with_network", 1), ("network_off", 0)):
        sim.learned_enable(on)
        for _ in range(args.warmup):
            sim.step(1)
        ms = C.c_double(0)
        if lib.icep_step_timed(sim.ctx, args.steps, C.byref(ms)) != 0:
            raise RuntimeError("learned timed steps failed")
        it, err, _ = sim.solver_stats()
        fb, apps = sim.learned_stats()
        v = args.steps / (ms.value / 1000.0)
        out[key] = {"value": v, "unit": UNIT, "ms_per_step": ms.value / args.steps, "vs_plain": v / plain_value,
                    "inner_iterations_last_solve": it, "network_applications_last_solve": apps if on else 0,
                    "fallbacks_last_solve": fb, "relative_true_residual": err}
    sim.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--np", type=int, default=512)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--maxit", type=int, default=1000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
    else:
        run_gpu(args, world, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
