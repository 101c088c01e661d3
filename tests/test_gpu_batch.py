"""Batches of independent replicas (icep_batch_*): replicas advanced together
on their own streams give the results of the same replicas advanced alone
(MIXED precision; tolerances as for repeated runs: the particle scatters use
atomics, so the summation order may differ between runs)."""
import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi
from icep_kapsel_gb300.runtime import Batch, IcepError, Simulation

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


def replica(n, npart, seed, ez):
    return cases.icep_case(n=n, npart=npart, minsep=10.0, seed=seed, a=4.0, eps_f=80.0, eps_p=3.0,
                           e_ext=(0.0, 0.0, ez), tol=1e-8, maxit=1000, dt=0.01, per_particle_eps=(1.0, 5.0),
                           solver=abi.SOLVER_SPECTRAL, precision=abi.MIXED)


def test_batch_matches_single_replicas():
    specs = [(32, 6, 1, 0.05), (64, 20, 2, 0.1), (32, 8, 3, 0.2), (64, 12, 4, 0.15)]
    b = Batch([replica(*sp) for sp in specs])
    b.init_state()
    b.step(3)
    for i, sp in enumerate(specs):
        s = Simulation(*replica(*sp))
        s.init_state()
        s.step(3)
        r = b.replica(i)
        for name in ("zeta0", "zeta1", "phi", "c0"):
            assert rel(r.get(name), s.get(name)) < 1e-5, (i, name)
        xa = np.array([[q.x[d] for d in range(3)] for q in r.particles()[:sp[1]]])
        xb = np.array([[q.x[d] for d in range(3)] for q in s.particles()[:sp[1]]])
        assert rel(xa, xb) < 1e-9
        s.close()
    b.close()


def test_batch_create_reports_a_bad_replica():
    good = replica(32, 6, 1, 0.1)
    p, parts = replica(32, 6, 2, 0.1)
    p.nx = 48  # not a power of two
    with pytest.raises(IcepError):
        Batch([good, (p, parts)])
