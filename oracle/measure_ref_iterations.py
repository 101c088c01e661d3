#!/usr/bin/env python3
"""Per-step iteration counts of the reference Poisson solve on the bench
workload (128^3, 512 spheres, eps_p uniform in [1, 5], eps_f = 80,
E0 = (0, 0, 0.1), tol 1e-8, MaxIter 1000): the oracle's restatement of
Charge_field2potential_dielectric_LO (identity-preconditioned BiCGSTAB with
the MaxIter retry, operate_dielectric.cxx:542-572), FP64, all host threads.
matvecs counts every operator application of the step's solve (initial
residual, restarts and a MaxIter retry included).

Writes oracle/ref_iterations_128.json, which the CPU reference arm of
bench.py combines with live per-iteration timings: a full step of the
reference takes minutes on a CPU, so the arm times a capped step and one
iteration and composes each step's time from the recorded counts.

    python oracle/measure_ref_iterations.py [--steps 16]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (ROOT, os.path.join(ROOT, "tests"), HERE):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--out", default=os.path.join(HERE, "ref_iterations_128.json"))
    a = ap.parse_args()
    import cases
    import pyoracle
    from icep_kapsel_gb300 import abi
    p, parts = cases.icep_case(n=128, npart=512, minsep=10.0, seed=2024, a=4.0, eps_f=80.0, eps_p=3.0,
                               e_ext=(0.0, 0.0, 0.1), tol=1e-8, maxit=1000, dt=0.01, per_particle_eps=(1.0, 5.0),
                               solver=abi.SOLVER_REF, precision=abi.FP64)
    o = pyoracle.Oracle(p, parts)
    rec = {"workload": "icep_step_128^3_512_spheres", "solver": "reference BiCGSTAB (identity), MaxIter retry",
           "tol": 1e-8, "maxit": 1000, "threads": int(o.lib.ko_max_threads()), "init": None, "steps": []}
    t0 = time.time()
    m0 = o.matvecs()
    o.init_state()
    rec["init"] = {"iterations": o.last_iterations(), "matvecs": o.matvecs() - m0, "rel_residual": o.last_error(),
                   "s": time.time() - t0}
    print("init", rec["init"], flush=True)
    for k in range(a.steps):
        t0 = time.time()
        m0 = o.matvecs()
        o.step(1)
        e = {"iterations": o.last_iterations(), "matvecs": o.matvecs() - m0, "rel_residual": o.last_error(),
             "s": time.time() - t0}
        rec["steps"].append(e)
        print(k + 1, e, flush=True)
        with open(a.out, "w") as fh:
            json.dump(rec, fh, indent=1)


if __name__ == "__main__":
    main()
