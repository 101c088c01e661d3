"""Checkpoint / restart (icep_save_checkpoint / icep_load_checkpoint; the
reference's Save_Restart_udf and Force_restore_parameters, resume.cxx:10-78,
308-398, plus the potential).

A run that saves after k steps and a fresh context that loads the file must
continue exactly as the uninterrupted run: bit-identical up to the order of
the atomics in the particle scatters (FP64: 1e-12; MIXED: 1e-6 relative,
the FP32 rounding of those sums). A file for another mesh is refused, and a
truncated file leaves the context unchanged.
"""
import os

import numpy as np
import pytest

import cases
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


def icep(precision, n=32):
    return cases.icep_case(n=n, npart=4, minsep=12.0, seed=2, eps_f=80.0, eps_p=3.0, e_ext=(0.0, 0.0, 0.1),
                           tol=1e-8, solver=abi.SOLVER_SPECTRAL, precision=precision)


def state(s, electrolyte=True):
    keys = ("zeta0", "zeta1", "c0", "c1", "pot") if electrolyte else ("zeta0", "zeta1")
    out = {k: s.get(k) for k in keys}
    pa = abi.particles_to_numpy(s.particles(), s.params.n_particles)
    out["x"], out["v"] = pa["x"], pa["v"]
    return out


@pytest.mark.parametrize("precision,tol", [(abi.FP64, 1e-12), (abi.MIXED, 1e-6)])
def test_restart_continues_the_run(Sim, tmp_path, precision, tol):
    path = str(tmp_path / "run.ckpt")
    p, parts = icep(precision)
    a = Sim(p, parts)
    a.init_state()
    a.step(3)
    a.save_checkpoint(path)
    assert os.path.getsize(path) > 0
    a.step(2)
    ref = state(a)
    p2, parts2 = icep(precision)
    b = Sim(p2, parts2)  # fresh context, no init_state: the file is the whole state
    b.load_checkpoint(path)
    assert b.time()[0] == 3
    assert abs(b.time()[1] - 3 * p.dt) < 1e-15
    b.step(2)
    got = state(b)
    assert b.time() == a.time()
    for k in ref:
        v, w = got[k], ref[k]
        if k == "pot":
            nz = p.nz
            v, w = v[:, :, :nz] - v[:, :, :nz].mean(), w[:, :, :nz] - w[:, :, :nz].mean()
        assert rel(v, w) < tol, k


def test_restart_navier_stokes(Sim, tmp_path):
    path = str(tmp_path / "ns.ckpt")
    x = cases.positions(4, 32, 12.0, 3)
    p = abi.make_params(nx=32, ny=32, nz=32, n_particles=4, dt=0.05, janus_propulsion=[abi.MOTOR],
                        janus_force=[[0.01, 0.0, 0.0]])
    a = Sim(p, abi.make_particles(x))
    a.init_state()
    a.step(5)
    a.save_checkpoint(path)
    a.step(5)
    b = Sim(p, abi.make_particles(x))
    b.load_checkpoint(path)
    b.step(5)
    ra, rb = state(a, False), state(b, False)
    for k in ra:
        assert rel(rb[k], ra[k]) < 1e-12, k


def test_restart_refuses_mismatch_and_truncation(Sim, tmp_path):
    from icep_kapsel_gb300.runtime import IcepError
    path = str(tmp_path / "a.ckpt")
    p, parts = icep(abi.FP64)
    a = Sim(p, parts)
    a.init_state()
    a.step(1)
    a.save_checkpoint(path)
    p64, parts64 = icep(abi.FP64, n=64)
    c = Sim(p64, parts64)
    with pytest.raises(IcepError):
        c.load_checkpoint(path)
    bad = str(tmp_path / "short.ckpt")
    with open(path, "rb") as fh:
        blob = fh.read()
    with open(bad, "wb") as fh:
        fh.write(blob[: len(blob) // 2])
    before = state(a)
    with pytest.raises(IcepError):
        a.load_checkpoint(bad)
    after = state(a)
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    with pytest.raises(IcepError):
        a.load_checkpoint(str(tmp_path / "missing.ckpt"))
