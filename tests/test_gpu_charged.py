"""Charged particles in the salt solution on the GPU (Init_rho_ion's
counterions, Conc_k2charge_field with Make_phi_qq_particle; the surface-charge
branch of Init_potential_dielectric and Make_Maxwell_force_x_on_fluid).

* FP64 against the golden fixture made with the reference's own code
  (tests/golden/charged32: concentrations 1e-13, charge field and Phi sum
  1e-13 -- atomics add in a different order; initial potential 2e-5, the
  reference's BiCGSTAB iterate at its 1e-7 tolerance).
* FP64 with the spectral solver against the oracle for two steps (1e-8).
* MIXED against FP64 (the tolerances of test_gpu_mixed.py).
* Charged and uncharged species together are refused.
* INIT_profile Poisson_Boltzmann: the relaxed initial densities against the
  reference's relaxation (tests/golden/charged32_pb, 1e-12); the branches that
  are not built are refused.
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


def test_charged_against_reference_golden(Sim):
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "charged32.npz"))
    p, parts = cases.charged_case()
    s = Sim(p, parts)
    s.init_state()
    for k in ("c0", "c1"):
        assert rel(s.get(k), g[k]) < 1e-13, k
    a = s.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    s.call("charge_field")
    assert rel(s.get("rho")[:, :, :32], g["rho"]) < 1e-13
    assert rel(s.get("work")[:, :, :32], g["phi_p"]) < 1e-13


def test_charged_spectral_steps_against_oracle(Sim):
    p, parts = cases.charged_case(charges=(-5.0, -2.0), tol=1e-10, solver=abi.SOLVER_SPECTRAL)
    s = Sim(p, parts)
    o = pyoracle.Oracle(p, parts)
    s.init_state(); o.init_state()
    s.step(2); o.step(2)
    nz = p.nz
    a, b = s.get("pot")[:, :, :nz], o.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 1e-8
    for k in ("zeta0", "zeta1", "c0", "c1"):
        assert rel(s.get(k), o.get(k)) < 1e-8, k
    pa = abi.particles_to_numpy(s.particles(), p.n_particles)
    pb = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["x"], pb["x"]) < 1e-12


def test_charged_mixed_against_fp64(Sim):
    pm, parts = cases.charged_case(n=64, npart=16, charges=(-5.0,), tol=1e-8, solver=abi.SOLVER_SPECTRAL,
                                   precision=abi.MIXED, eps_f=80.0, eps_p=3.0, e_ext=(0.0, 0.0, 0.1))
    pd, parts_d = cases.charged_case(n=64, npart=16, charges=(-5.0,), tol=1e-8, solver=abi.SOLVER_SPECTRAL,
                                     precision=abi.FP64, eps_f=80.0, eps_p=3.0, e_ext=(0.0, 0.0, 0.1))
    m = Sim(pm, parts)
    d = Sim(pd, parts_d)
    m.init_state(); d.init_state()
    m.step(3); d.step(3)
    _, err, _ = m.solver_stats()
    assert err <= 1e-8
    nz = pm.nz
    a, b = m.get("pot")[:, :, :nz], d.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 2e-5
    for k in ("zeta0", "zeta1"):
        assert rel(m.get(k), d.get(k)) < 1e-3, k
    for k in ("c0", "c1"):
        assert rel(m.get(k), d.get(k)) < 1e-5, k


def test_mixed_charged_and_neutral_species_refused(Sim):
    from icep_kapsel_gb300.runtime import IcepError
    p, parts = cases.charged_case(charges=(-5.0, 0.0))
    with pytest.raises(IcepError):
        Sim(p, parts)


def test_poisson_boltzmann_init_against_reference_golden(Sim):
    """INIT_profile Poisson_Boltzmann (Init_rho_ion -> Set_steadystate_ion_density,
    operate_electrolyte.cxx:424-457, 834-853): FP64 GPU relaxation of the salt
    densities in the external field against the reference's own relaxation
    (tests/golden/charged32_pb): the densities within 1e-12 (the relaxation
    stops at the same step of its free-energy test), the initial potential
    within the reference BiCGSTAB's 1e-7 tolerance (2e-5); the relaxed
    densities differ from the uniform start."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "charged32_pb.npz"))
    p, parts = cases.pb_case()
    s = Sim(p, parts)
    s.init_state()
    for k in ("c0", "c1"):
        assert rel(s.get(k), g[k]) < 1e-12, k
    a = s.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    u, uparts = cases.charged_case(e_ext=(0.0, 0.0, 0.1))
    uni = Sim(u, uparts)
    uni.init_state()
    assert rel(uni.get("c0"), g["c0"]) > 1e-3
    s.step(2)  # the step runs on from the relaxed state
    assert np.isfinite(s.get("c0")).all()


def test_poisson_boltzmann_unbuilt_branches_refused(Sim):
    """The salt-free and single-particle relaxations are refused, not run."""
    from icep_kapsel_gb300.runtime import IcepError
    p, parts = cases.saltfree_case()
    p.poisson_boltzmann = 1
    with pytest.raises(IcepError):
        Sim(p, parts)
    q, qparts = cases.charged_case(npart=1)
    q.poisson_boltzmann = 1
    with pytest.raises(IcepError):
        Sim(q, qparts)
