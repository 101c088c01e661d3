"""Salt-free electrolyte on the GPU (Add_salt saltfree, N_spec = 1: the
counterions of the charged particles only; Init_rho_ion with
Set_uniform_ion_charge_density_nosalt, operate_electrolyte.cxx:738-862,
459-493).

* FP64 against the reference-generated fixture saltfree32: the counterion
  density 1e-13, the charge field 1e-12, the initial potential 2e-5 (the
  reference's BiCGSTAB iterate at its 1e-7 tolerance); the absent second
  species is zero.
* FP64 with the spectral solver against the oracle for three steps (1e-8);
  the second concentration stays exactly zero.
* MIXED against FP64 at 64^3 (the tolerances of test_gpu_mixed.py).
* Refused: uncharged particles, particles of both signs, a counterion
  valency of the particles' sign.
"""
import os

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


def test_saltfree_against_reference_golden(Sim):
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "saltfree32.npz"))
    p, parts = cases.saltfree_case()
    s = Sim(p, parts)
    s.init_state()
    assert rel(s.get("c0"), g["c0"]) < 1e-13
    assert np.abs(s.get("c1")).max() == 0.0
    a = s.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    s.call("charge_field")
    assert rel(s.get("rho")[:, :, :32], g["rho"]) < 1e-12


def test_saltfree_spectral_steps_against_oracle(Sim):
    p, parts = cases.saltfree_case(tol=1e-10, solver=abi.SOLVER_SPECTRAL)
    s = Sim(p, parts)
    o = pyoracle.Oracle(p, parts)
    s.init_state()
    o.init_state()
    s.step(3)
    o.step(3)
    nz = p.nz
    a, b = s.get("pot")[:, :, :nz], o.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 1e-8
    for k in ("zeta0", "zeta1", "c0"):
        assert rel(s.get(k), o.get(k)) < 1e-8, k
    assert np.abs(s.get("c1")).max() == 0.0
    pa = abi.particles_to_numpy(s.particles(), p.n_particles)
    pb = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["x"], pb["x"]) < 1e-12


def test_saltfree_mixed_against_fp64(Sim):
    def case(precision):
        p, _ = cases.saltfree_case(tol=1e-8, solver=abi.SOLVER_SPECTRAL, precision=precision)
        p.nx = p.ny = p.nz = 64
        p.n_particles = 16
        x = cases.positions(16, 64, 12.0, 3)
        return p, abi.make_particles(x, spec=[i % 2 for i in range(16)])
    pm, parts_m = case(abi.MIXED)
    pd, parts_d = case(abi.FP64)
    m = Sim(pm, parts_m)
    d = Sim(pd, parts_d)
    m.init_state()
    d.init_state()
    m.step(3)
    d.step(3)
    _, err, _ = m.solver_stats()
    assert err <= 1e-8
    nz = pm.nz
    a, b = m.get("pot")[:, :, :nz], d.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 2e-5
    for k in ("zeta0", "zeta1"):
        assert rel(m.get(k), d.get(k)) < 1e-3, k
    assert rel(m.get("c0"), d.get("c0")) < 1e-5
    assert np.abs(m.get("c1")).max() == 0.0


@pytest.mark.parametrize("charges,valency", [((0.0,), 1.0), ((-5.0, 3.0), 1.0), ((-5.0,), -1.0)])
def test_saltfree_refused(Sim, charges, valency):
    from icep_kapsel_gb300.runtime import IcepError
    p, parts = cases.saltfree_case(charges=charges, valency=valency)
    with pytest.raises(IcepError):
        Sim(p, parts)


def test_saltfree_dropin_one_concentration(Sim):
    """The drop-in call of a salt-free run takes one concentration array
    (conc1 NULL) and continues the device-resident run (1e-12, FP64)."""
    p, parts = cases.saltfree_case(tol=1e-10, solver=abi.SOLVER_SPECTRAL)
    a = Sim(p, parts)
    a.init_state()
    a.step(1)
    q, qparts = cases.saltfree_case(tol=1e-10, solver=abi.SOLVER_SPECTRAL)
    b = Sim(q, qparts)
    b.init_state()
    b.step(1)
    host = {k: np.ascontiguousarray(b.get(k)) for k in ("zeta0", "zeta1", "c0", "pot")}
    uk = np.ascontiguousarray(b.uk_dc())
    hp = b.particles()
    for _ in range(2):
        b.time_evolution(host["zeta0"], host["zeta1"], uk, hp, host["c0"], None, host["pot"], 1)
    a.step(2)
    for k in ("zeta0", "zeta1", "c0"):
        assert rel(host[k], a.get(k)) < 1e-12, k
    assert np.abs(b.get("c1")).max() == 0.0
