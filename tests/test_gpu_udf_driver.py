"""The command-line driver (icep_kapsel -I input.udf) on the GPU: it runs
GTS * Num_snap steps of the UDF fixture, writes a particle file every GTS
steps and a restart checkpoint, and its result equals the same run made
through the Python API from icep_udf_read's parameters (FP64: 1e-12, the
order of the scatter atomics)."""
import os
import subprocess

import numpy as np
import pytest

from icep_kapsel_gb300 import abi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "udf", "input_small.udf")


@pytest.fixture(scope="module")
def rt():
    from icep_kapsel_gb300 import build
    build.build()
    from icep_kapsel_gb300 import runtime
    return runtime


def test_driver_matches_api(rt, tmp_path):
    from icep_kapsel_gb300.build import BIN
    out = str(tmp_path / "out")
    r = subprocess.run([BIN, "-I", FIX, "-O", out, "--solver", "spectral"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "poisson iterations" in r.stderr
    files = sorted(f for f in os.listdir(out) if f.startswith("particles_"))
    assert files == ["particles_00000000.dat", "particles_00000002.dat", "particles_00000004.dat"]
    got = np.loadtxt(os.path.join(out, files[-1]))
    p, parts, gts, nsnap = rt.udf_read(FIX)
    p.solver = abi.SOLVER_SPECTRAL
    s = rt.Simulation(p, parts)
    s.init_state()
    s.step(gts * nsnap)
    a = abi.particles_to_numpy(s.particles(), p.n_particles)
    ref = np.hstack([a["spec"][:, None], a["x"], a["v"], a["omega"], a["q"]])
    assert np.array_equal(got[:, 0], ref[:, 0])
    nb = np.linalg.norm(ref[:, 1:4])
    assert np.linalg.norm(got[:, 1:4] - ref[:, 1:4]) / nb < 1e-12
    assert np.linalg.norm(got[:, 4:7] - ref[:, 4:7]) <= 1e-10 * max(np.linalg.norm(ref[:, 4:7]), 1e-30)
    # the checkpoint restores the same state into a fresh context
    c = rt.Simulation(p, parts)
    c.load_checkpoint(os.path.join(out, "restart.ckpt"))
    assert c.time()[0] == gts * nsnap
    for k in ("zeta0", "zeta1", "c0", "c1"):
        v, w = c.get(k), s.get(k)
        assert np.linalg.norm(v - w) <= 1e-10 * np.linalg.norm(w), k


def test_driver_refuses_unsupported(rt, tmp_path):
    from icep_kapsel_gb300.build import BIN
    src = open(FIX).read().replace('{"ON", {1000, 1.0e-8, 80.0, 5.0, 2.0}}', '{"OFF", {1000, 1.0e-8, 80.0, 5.0, 2.0}}')
    d = tmp_path / "u"
    d.mkdir()
    (d / "define_small.udf").write_text(open(os.path.join(os.path.dirname(FIX), "define_small.udf")).read())
    (d / "input.udf").write_text(src)
    r = subprocess.run([BIN, "-I", str(d / "input.udf"), "-O", str(tmp_path / "o")], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 3  # ICEP_ERR_UNSUPPORTED
    assert "Dielectric_property OFF" in r.stderr
