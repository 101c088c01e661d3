"""The step as one CUDA graph (icep_step_graphs): the MIXED Poisson solve's
refinement sweeps and inner iterations run as device-side loops (conditional
WHILE nodes) and the whole step replays as one launch, alone or for every
replica of a batch at once. Its results are the host-driven step's: the same
kernels in the same order with the same scalars (formed on the device in the
host loop's double arithmetic), so fields agree to the run-to-run level of
the particle scatters' atomics and the solves take the same iterations.
"""
import os

import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi
from icep_kapsel_gb300.runtime import Batch, Simulation

pytestmark = pytest.mark.gpu

FIELDS = ("zeta0", "zeta1", "pot", "c0", "c1", "phi")


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


def replica(n, npart, seed, ez, a=4.0):
    return cases.icep_case(n=n, npart=npart, minsep=10.0, seed=seed, a=a, eps_f=80.0, eps_p=3.0,
                           e_ext=(0.0, 0.0, ez), tol=1e-8, maxit=1000, dt=0.01, per_particle_eps=(1.0, 5.0),
                           solver=abi.SOLVER_SPECTRAL, precision=abi.MIXED)


def host_driven(p, parts):
    """A context whose steps run without graphs (ICEP_GRAPHS=0 at creation)."""
    old = os.environ.get("ICEP_GRAPHS")
    os.environ["ICEP_GRAPHS"] = "0"
    try:
        return Simulation(p, parts)
    finally:
        if old is None:
            del os.environ["ICEP_GRAPHS"]
        else:
            os.environ["ICEP_GRAPHS"] = old


def positions(sim, n):
    return np.array([[q.x[d] for d in range(3)] for q in sim.particles()[:n]])


def compare(a, b, npart):
    for name in FIELDS:
        assert rel(a.get(name), b.get(name)) < 1e-5, name
    assert rel(positions(a, npart), positions(b, npart)) < 1e-9
    ita, era, _ = a.solver_stats()
    itb, erb, _ = b.solver_stats()
    assert abs(ita - itb) <= 1 and era <= 1e-8 and erb <= 1e-8, (ita, itb, era, erb)


def test_step_graph_matches_host_loop():
    p, parts = replica(64, 20, 2, 0.1)
    g = Simulation(p, parts)
    h = host_driven(*replica(64, 20, 2, 0.1))
    for s in (g, h):
        s.init_state()
        s.step(5)
    # the first step (Euler integrators) runs as before, the next four as graphs
    assert g.step_graphs() == 4 and h.step_graphs() == 0
    compare(g, h, 20)
    g.close()
    h.close()


def test_batch_graph_matches_host_driven_replicas():
    """Uneven replicas (meshes 32^3 and 64^3, 6-20 spheres, different fields):
    every batch step after the first is one graph launch for all of them."""
    specs = [(32, 6, 1, 0.05), (64, 20, 2, 0.1), (32, 8, 3, 0.2), (64, 12, 4, 0.15)]
    b = Batch([replica(*sp) for sp in specs])
    b.init_state()
    b.step(4)
    for i, sp in enumerate(specs):
        r = b.replica(i)
        assert r.step_graphs() == 3, i
        h = host_driven(*replica(*sp))
        h.init_state()
        h.step(4)
        compare(r, h, sp[1])
        h.close()
    b.close()


def test_step_graph_zero_right_hand_side():
    """No external field and neutral uniform ions: b = 0 every step, the sweep
    loop does not run and the potential is zero, as on the host path."""
    p, parts = replica(32, 6, 5, 0.0)
    g = Simulation(p, parts)
    h = host_driven(*replica(32, 6, 5, 0.0))
    for s in (g, h):
        s.init_state()
        s.step(3)
    assert g.step_graphs() == 2
    for s in (g, h):
        it, er, _ = s.solver_stats()
        assert it == 0 and np.abs(s.get("pot")).max() == 0.0
    for name in ("zeta0", "zeta1", "phi", "c0"):
        assert rel(g.get(name), h.get(name)) < 1e-5, name
    g.close()
    h.close()


def with_inner(solver, p, parts):
    """A context whose MIXED inner solve is `solver` (ICEP_INNER at creation)."""
    old = os.environ.get("ICEP_INNER")
    os.environ["ICEP_INNER"] = solver
    try:
        return Simulation(p, parts)
    finally:
        if old is None:
            del os.environ["ICEP_INNER"]
        else:
            os.environ["ICEP_INNER"] = old


def test_inner_cg_and_bicgstab_agree():
    """The inner correction solve by preconditioned CG (the default) or by
    BiCGSTAB: both sweeps end at the same true-residual criterion, so the
    steps agree to the solve tolerance; CG takes one operator application
    per iteration, BiCGSTAB two."""
    sims = {k: with_inner(k, *replica(64, 20, 2, 0.1)) for k in ("cg", "bicgstab")}
    for s in sims.values():
        s.init_state()
        s.step(4)
    a, b = sims["cg"], sims["bicgstab"]
    for name in ("zeta0", "zeta1", "c0", "phi"):
        assert rel(a.get(name), b.get(name)) < 1e-5, name
    assert rel(a.get("pot"), b.get("pot")) < 2e-5
    ita, era, mva = a.solver_stats()
    itb, erb, mvb = b.solver_stats()
    assert era <= 1e-8 and erb <= 1e-8
    assert 0 < ita <= 2 * itb + 2, (ita, itb)
    for s in sims.values():
        s.close()
