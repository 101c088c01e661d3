"""Janus dielectric particles (Make_janus_permittivity_dielectric,
operate_dielectric.cxx:173-292) on the GPU.

* FP64: the permittivity field and the phi_sin sum against the oracle
  (1e-13; atomics add in a different order), then two ICEP steps with the
  spectral solver (1e-8, as for the other FP64 operator tests).
* MIXED against FP64 on the same case (the tolerances of test_gpu_mixed.py).
* Argument checks: a Janus field with per-particle permittivity, or with a
  particle whose species has no axis, is refused (the reference exits).
"""
import numpy as np
import pytest

import cases
import pyoracle
from icep_kapsel_gb300 import abi

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="module")
def Sim():
    from icep_kapsel_gb300.build import build
    build()
    from icep_kapsel_gb300.runtime import Simulation
    return Simulation


def case(precision, n=32, npart=6):
    return cases.janus_case(n=n, npart=npart, axes=(abi.JANUS_Z, abi.JANUS_X), eps_f=4.0, tol=1e-10,
                            solver=abi.SOLVER_SPECTRAL, precision=precision)


def test_janus_fp64_against_oracle(Sim):
    p, parts = case(abi.FP64)
    g = Sim(p, parts)
    o = pyoracle.Oracle(p, parts)
    g.init_state()
    o.init_state()
    nz = p.nz
    assert rel(g.get("eps")[:, :, :nz], o.get("eps")[:, :, :nz]) < 1e-13
    g.step(2)
    o.step(2)
    assert rel(g.get("eps")[:, :, :nz], o.get("eps")[:, :, :nz]) < 1e-13
    a, b = g.get("pot")[:, :, :nz], o.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 1e-8
    for k in ("zeta0", "zeta1", "c0", "c1"):
        assert rel(g.get(k), o.get(k)) < 1e-8, k
    pa = abi.particles_to_numpy(g.particles(), p.n_particles)
    pb = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["x"], pb["x"]) < 1e-12


def test_janus_mixed_against_fp64(Sim):
    pm, parts = case(abi.MIXED, n=64, npart=24)
    pd, parts_d = case(abi.FP64, n=64, npart=24)
    pm.potential_tol = pd.potential_tol = 1e-8
    m = Sim(pm, parts)
    d = Sim(pd, parts_d)
    m.init_state()
    d.init_state()
    nz = pm.nz
    assert rel(m.get("eps")[:, :, :nz], d.get("eps")[:, :, :nz]) < 1e-6
    m.step(3)
    d.step(3)
    _, err, _ = m.solver_stats()
    assert err <= 1e-8
    a, b = m.get("pot")[:, :, :nz], d.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 2e-5
    for k in ("zeta0", "zeta1"):
        assert rel(m.get(k), d.get(k)) < 1e-3, k


def test_janus_argument_checks(Sim):
    from icep_kapsel_gb300.runtime import IcepError
    p, parts = case(abi.FP64)
    p.per_particle_eps = 1
    with pytest.raises(IcepError):
        Sim(p, parts)
    p, parts = case(abi.FP64)
    p.janus_axis[1] = abi.JANUS_NONE  # species 1 (odd particles) without an axis
    with pytest.raises(IcepError):
        Sim(p, parts)
