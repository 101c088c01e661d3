"""Field output on the GPU: icep_charge_field_data (the fields of
Output_dielectric_charge_field_data, output.cxx:262-320) and
icep_output_avs (the reference's AVS frames of the context's state).

* FP64 against the reference-generated fixture out32 (the charged case after
  its initial solve, with zeta from icep32_bicgstab and a mean flow): u 1e-12, phi and
  the surface charge 1e-13 (scatter atomics add in another order), the
  solute charge 1e-12, eps 1e-13; the potential is the context's own.
* MIXED against the same fixture at FP32 tolerances (2e-6; the solute
  charge 1e-5: FP32 FFTs of the concentrations).
* The output leaves the step state alone: a run that writes output every
  step matches one that does not (1e-12, FP64).
* Uncharged particles give a NaN surface charge (0/0), as the reference.
* icep_output_avs writes what icep_charge_field_data returns (float32) and
  the particle positions, under the headers of icep_avs_init; the driver
  writes a frame every GTS steps when the input turns AVS output on.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import cases
from icep_kapsel_gb300 import abi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
FIX = os.path.join(HERE, "golden", "udf", "input_small.udf")


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


@pytest.fixture(scope="module")
def Sim():
    from icep_kapsel_gb300.build import build
    build()
    from icep_kapsel_gb300.runtime import Simulation
    return Simulation


def out32_state(Sim, precision):
    ic = np.load(os.path.join(GOLD, "icep32_bicgstab.npz"))
    p, parts = cases.charged_case()
    p.precision = precision
    p.solver = abi.SOLVER_SPECTRAL
    s = Sim(p, parts)
    s.init_state()
    s.set("zeta0", ic["zeta0"])
    s.set("zeta1", ic["zeta1"])
    s.set_uk_dc(np.array([30.0, -60.0, 15.0]))
    return s


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_charge_field_data_against_reference(Sim, precision):
    g = np.load(os.path.join(GOLD, "out32.npz"))
    s = out32_state(Sim, precision)
    o = s.charge_field_data()
    t = 1e-12 if precision == abi.FP64 else 2e-6
    for k in ("u0", "u1", "u2"):
        assert rel(o[k][:, :, :32], g[k]) < t, k
    assert rel(o["phi"][:, :, :32], g["phi"]) < (1e-13 if precision == abi.FP64 else 2e-6)
    assert rel(o["surface_charge"][:, :, :32], g["up0"]) < (1e-13 if precision == abi.FP64 else 2e-6)
    assert rel(o["solute_charge"][:, :, :32], g["up1"]) < (1e-12 if precision == abi.FP64 else 1e-5)
    assert rel(o["epsilon"][:, :, :32], g["up2"]) < (1e-13 if precision == abi.FP64 else 2e-6)
    assert np.array_equal(o["potential"], s.get("pot"))


def test_output_leaves_state(Sim):
    a = out32_state(Sim, abi.FP64)
    b = out32_state(Sim, abi.FP64)
    for _ in range(2):
        a.charge_field_data()
        a.step(1)
        b.step(1)
    for k in ("zeta0", "zeta1", "c0", "c1", "pot"):
        assert rel(a.get(k), b.get(k)) < 1e-12, k


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_uncharged_surface_is_nan(Sim, precision):
    p, parts = cases.icep_case(solver=abi.SOLVER_SPECTRAL, precision=precision)
    s = Sim(p, parts)
    s.init_state()
    o = s.charge_field_data()
    assert np.all(np.isnan(o["surface_charge"][:, :, :32]))
    assert np.all(np.isfinite(o["solute_charge"][:, :, :32]))


def test_output_avs_frame(Sim, tmp_path):
    s = out32_state(Sim, abi.FP64)
    d = str(tmp_path / "avs")
    s.avs_init(d, "data", nstep=3)
    s.output_avs(d, "data")
    o = s.charge_field_data()
    ts, _ = s.time()
    data = np.fromfile(os.path.join(d, "avs", "data_%d.dat" % ts), dtype=np.float32).reshape(7, 32, 32, 32)
    keys = ("u0", "u1", "u2", "phi", "surface_charge", "solute_charge", "potential")
    for v, k in enumerate(keys):
        ref = o[k][:, :, :32].astype(np.float32).transpose(2, 1, 0)
        assert np.allclose(data[v], ref, rtol=1e-6, atol=0), k
    n = s.params.n_particles
    cod = np.fromfile(os.path.join(d, "avs", "datap_%d.cod" % ts), dtype=np.float32).reshape(3, n)
    x = abi.particles_to_numpy(s.particles(), n)["x"]
    assert np.array_equal(cod, x[:, ::-1].T.astype(np.float32))
    fld = open(os.path.join(d, "data.fld")).read()
    assert 'time value = "step%dtime' % ts in fld and fld.rstrip().endswith("EOT")


def test_driver_writes_avs_frames(tmp_path):
    from icep_kapsel_gb300.build import BIN
    d = tmp_path / "udf"
    d.mkdir()
    with open(os.path.join(os.path.dirname(FIX), "define_small.udf")) as fh:
        (d / "define_small.udf").write_text(fh.read())
    src = open(FIX).read().replace('output:{2, 2, "OFF", {"avs_out", "data", "BINARY"}}',
                                   'output:{2, 2, "ON", {"avs_out", "data", "BINARY"}}')
    (d / "input.udf").write_text(src)
    r = subprocess.run([BIN, "-I", str(d / "input.udf"), "-O", str(tmp_path / "out"), "--solver", "spectral"],
                       capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    avs = tmp_path / "avs_out"
    names = sorted(os.listdir(avs / "avs"))
    assert names == ["data_0.dat", "data_2.dat", "data_4.dat", "datap_0.cod", "datap_0.dat", "datap_2.cod",
                     "datap_2.dat", "datap_4.cod", "datap_4.dat"]
    fld = (avs / "data.fld").read_text()
    assert "nstep=3" in fld and fld.count("EOT") == 3
    assert os.path.getsize(avs / "avs" / "data_4.dat") == 7 * 4 * 32 ** 3
