"""An AC external field, E_ext sin(2 pi f t) (Electric_field.ON.AC), on the GPU.

* FP64 with the reference's solver against the reference-generated golden
  fixture ac32 (the tolerances of the DC fixture icep32_bicgstab): the field is zero at
  t = 0, so the first step's potential is exactly zero, and the next two steps
  run with the field at t = dt and 2 dt.
* FP64 with the spectral solver against the oracle over four steps (1e-8).
* MIXED against FP64 on a 64^3 case (the tolerances of test_gpu_mixed.py).
* A checkpoint carries the time: a run resumed from it continues the phase
  of the field (1e-12 in FP64).
"""
import json
import os

import numpy as np
import pytest

import cases
import pyoracle
from icep_kapsel_gb300 import abi

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="module")
def Sim():
    from icep_kapsel_gb300.build import build
    build()
    from icep_kapsel_gb300.runtime import Simulation
    return Simulation


def test_ac32_golden(Sim):
    g = np.load(os.path.join(GOLD, "ac32.npz"))
    with open(os.path.join(GOLD, "ac32.json")) as fh:
        meta = json.load(fh)
    p, parts = cases.ac_case()
    o = Sim(p, parts)
    o.init_state()
    o.step(1)
    assert meta["step0_iterations"] == 0
    assert np.abs(o.get("pot")[:, :, :32]).max() == 0.0
    o.step(2)
    for k in ("zeta0", "zeta1"):
        assert rel(o.get(k), g[k]) < 2e-5, k
    for k in ("c0", "c1"):
        assert rel(o.get(k), g[k]) < 1e-9, k
    a = o.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    pa = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["x"], g["p_x"]) < 1e-12
    assert rel(pa["v"], g["p_v"]) < 2e-5


def test_ac_spectral_fp64_against_oracle(Sim):
    p, parts = cases.ac_case(tol=1e-10, solver=abi.SOLVER_SPECTRAL)
    s = Sim(p, parts)
    o = pyoracle.Oracle(p, parts)
    s.init_state()
    o.init_state()
    s.step(4)
    o.step(4)
    nz = p.nz
    a, b = s.get("pot")[:, :, :nz], o.get("pot")[:, :, :nz]
    assert np.abs(b).max() > 0
    assert rel(a - a.mean(), b - b.mean()) < 1e-8
    for k in ("zeta0", "zeta1", "c0", "c1"):
        assert rel(s.get(k), o.get(k)) < 1e-8, k
    pa = abi.particles_to_numpy(s.particles(), p.n_particles)
    pb = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["x"], pb["x"]) < 1e-12


def test_ac_mixed_against_fp64(Sim):
    def case(precision):
        p, _ = cases.ac_case(tol=1e-8, solver=abi.SOLVER_SPECTRAL, precision=precision)
        p.nx = p.ny = p.nz = 64
        p.n_particles = 24
        x = cases.positions(24, 64, 12.0, 5)
        return p, abi.make_particles(x)
    pm, parts_m = case(abi.MIXED)
    pd, parts_d = case(abi.FP64)
    m = Sim(pm, parts_m)
    d = Sim(pd, parts_d)
    m.init_state()
    d.init_state()
    m.step(4)
    d.step(4)
    _, err, _ = m.solver_stats()
    assert err <= 1e-8
    nz = pm.nz
    a, b = m.get("pot")[:, :, :nz], d.get("pot")[:, :, :nz]
    assert rel(a - a.mean(), b - b.mean()) < 2e-5
    for k in ("zeta0", "zeta1"):
        assert rel(m.get(k), d.get(k)) < 1e-3, k
    for k in ("c0", "c1"):
        assert rel(m.get(k), d.get(k)) < 1e-6, k


def test_ac_checkpoint_keeps_phase(Sim, tmp_path):
    p, parts = cases.ac_case(tol=1e-10, solver=abi.SOLVER_SPECTRAL)
    a = Sim(p, parts)
    a.init_state()
    a.step(2)
    path = str(tmp_path / "ac.ckpt")
    a.save_checkpoint(path)
    a.step(2)
    q, qparts = cases.ac_case(tol=1e-10, solver=abi.SOLVER_SPECTRAL)
    b = Sim(q, qparts)
    b.load_checkpoint(path)
    b.step(2)
    nz = p.nz
    for k in ("zeta0", "zeta1", "c0", "c1"):
        assert rel(b.get(k), a.get(k)) < 1e-12, k
    x, y = b.get("pot")[:, :, :nz], a.get("pot")[:, :, :nz]
    assert rel(x - x.mean(), y - y.mean()) < 1e-12
