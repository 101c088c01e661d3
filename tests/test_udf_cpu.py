"""The UDF input front end (icep_udf_read / icep_udf_value; no GPU).

* The committed fixture tests/golden/udf/input_small.udf (+ its definitions):
  every key of the ICEP path lands in icep_params, user-specified particles
  with normalised quaternions, FIX_CELL bits, GTS / Num_snap.
* Settings outside the path are refused with ICEP_ERR_UNSUPPORTED, malformed
  files with ICEP_ERR_ARG, a short particle array with ICEP_ERR_ARG.
* When the reference tree is present: its own UDF/input.udf parses
  completely, and uniform_random placement reproduces libc's rand() sequence
  seeded with 10 (init_particle.cxx:18, macro.h:83-85).
"""
import ctypes as C
import os

import numpy as np
import pytest

from icep_kapsel_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "udf", "input_small.udf")
import pyoracle  # noqa: E402

REF_UDF = os.path.join(pyoracle.ref_dir(), "UDF", "input.udf")


@pytest.fixture(scope="module")
def rt():
    from icep_kapsel_gb300 import build
    build.build()
    from icep_kapsel_gb300 import runtime
    return runtime


def test_fixture_params(rt):
    p, parts, gts, nsnap = rt.udf_read(FIX)
    assert (p.nx, p.ny, p.nz) == (32, 32, 32)
    assert p.sw_eq == abi.ELECTROLYTE and p.dielectric == 1
    assert (p.dx, p.rho, p.eta, p.kbt, p.dt) == (1.0, 1.0, 1.0, 1.0, 0.01)
    assert (p.potential_iter, p.potential_tol) == (1000, 1e-8)
    assert (p.eps_fluid, p.eps_particle_top, p.eps_particle_bottom) == (80.0, 5.0, 2.0)
    assert (p.valency_pos, p.valency_neg, p.onsager_pos, p.onsager_neg, p.debye_length) == (1.0, -1.0, 7.24, 7.24, 10.0)
    assert p.external_field == 1 and list(p.e_ext) == [0.0, 0.0, 0.1]
    assert (p.a, p.a_xi, p.lj_epsilon, p.lj_powers, p.lj_truncate, p.rotation) == (4.0, 2.0, 1.0, 0, 1, 1)
    assert (p.g, p.g_direction) == (0.0, 2)
    assert p.n_species == 2 and list(p.janus_axis)[:2] == [abi.JANUS_Z, abi.JANUS_X]
    assert list(p.janus_propulsion)[:2] == [abi.NO_PROPULSION, abi.NO_PROPULSION]
    assert p.fix_cell == 4  # z only
    assert (p.precision, p.solver) == (abi.FP64, abi.SOLVER_REF)
    assert (gts, nsnap, p.n_particles) == (2, 2, 4)
    a = abi.particles_to_numpy(parts, 4)
    assert list(a["spec"]) == [0, 0, 1, 1]
    assert np.array_equal(a["x"][1], [24.0, 8.5, 8.0])
    assert np.array_equal(a["x_nopbc"], a["x"])
    # user quaternions normalised as qtn_normalize does: q * (1 / |q|)
    # (ROTATION ON, INIT_orientation user_specify)
    for i, q in ((1, [2.0, 0.0, 2.0, 0.0]), (3, [1.0, 1.0, 1.0, 1.0])):
        q = np.array(q)
        inv = 1.0 / np.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])
        assert np.array_equal(a["q"][i], q * inv)
    assert np.array_equal(a["q_old"], a["q"])


def test_fixture_values(rt):
    assert rt.udf_value(FIX, "mesh.NPY") == "5"
    assert rt.udf_value(FIX, "constitutive_eq.Electrolyte.Add_salt.saltfree.Onsager_coeff_counterion") == "7.24"
    assert rt.udf_value(FIX, "object_type.spherical_particle.Particle_spec.size") == "2"
    assert rt.udf_value(FIX, "switch.INIT_distribution.user_specify.Particles[2].R.z") == "20.0"
    with pytest.raises(rt.IcepError):
        rt.udf_value(FIX, "mesh.NPW")


def rewrite(tmp_path, old, new):
    src = open(FIX).read()
    assert old in src
    d = tmp_path / "udf"
    d.mkdir(exist_ok=True)
    with open(os.path.join(os.path.dirname(FIX), "define_small.udf")) as fh:
        (d / "define_small.udf").write_text(fh.read())
    (d / "input.udf").write_text(src.replace(old, new))
    return str(d / "input.udf")


def test_ac_field(rt, tmp_path):
    """Electric_field.ON.AC: E_ext and Frequency land in e_ext / frequency
    with ac = 1, and the auto time step takes a hundredth of the period when
    that is shorter than the viscous and diffusive times (input.cxx:369-375)."""
    path = rewrite(tmp_path, '{"ON", {"DC", {0.0, 0.0, 0.1}{0.0, 0.0, 0.0, 0.0}}}',
                   '{"ON", {"AC", {0.0, 0.0, 0.1}{0.0, 0.05, 0.1, 8.0}}}')
    p, _, _, _ = rt.udf_read(path)
    assert (p.external_field, p.ac, p.frequency) == (1, 1, 8.0)
    assert list(p.e_ext) == [0.0, 0.05, 0.1]
    assert p.dt == 0.01  # manual
    d = tmp_path / "udf"
    (d / "input.udf").write_text((d / "input.udf").read_text().replace(
        'time_increment:{"manual",{1.0}{0.01}}', 'time_increment:{"auto",{1.0}{0.01}}'))
    p, _, _, _ = rt.udf_read(str(d / "input.udf"))
    assert p.dt == 1.0 * (1.e-2 * (1. / 8.0))
    # the DC file keeps ac = 0
    p, _, _, _ = rt.udf_read(FIX)
    assert p.ac == 0


def test_saltfree(rt, tmp_path):
    """Add_salt saltfree: one ion species with the counterion valency and
    Onsager coefficient, which also sets the diffusive time of the auto time
    step (input.cxx:355-360)."""
    path = rewrite(tmp_path, '{"salt", {1.0, 7.24}{1.0, -1.0, 7.24, 7.24, 10.0}}',
                   '{"saltfree", {2.0, 3.5}{1.0, -1.0, 7.24, 7.24, 10.0}}')
    p, _, _, _ = rt.udf_read(path)
    assert (p.salt_free, p.valency_counterion, p.onsager_counterion) == (1, 2.0, 3.5)
    d = tmp_path / "udf"
    (d / "input.udf").write_text((d / "input.udf").read_text().replace(
        'time_increment:{"manual",{1.0}{0.01}}', 'time_increment:{"auto",{1.0}{0.01}}'))
    p, _, _, _ = rt.udf_read(str(d / "input.udf"))
    kmax2 = 3 * (2 * np.pi / 32 * 11) ** 2
    assert abs(p.dt - 1.0 / (1.0 * 3.5 * kmax2)) < 1e-15
    p, _, _, _ = rt.udf_read(FIX)
    assert p.salt_free == 0


def test_init_profile(rt, tmp_path):
    """INIT_profile (input.cxx:704-715): Uniform -> 0, Poisson_Boltzmann -> 1;
    any other word is an error."""
    p, _, _, _ = rt.udf_read(FIX)
    assert p.poisson_boltzmann == 0
    p, _, _, _ = rt.udf_read(rewrite(tmp_path, '"Uniform",', '"Poisson_Boltzmann",'))
    assert p.poisson_boltzmann == 1


@pytest.mark.parametrize("old,new", [
    ('{"ON", {1000, 1.0e-8, 80.0, 5.0, 2.0}}', '{"OFF", {1000, 1.0e-8, 80.0, 5.0, 2.0}}'),
    ('{"user_specify",\n', '{"uniform_random",\n'),  # fine: placement by rand()
])
def test_unsupported_or_changed(rt, tmp_path, old, new):
    path = rewrite(tmp_path, old, new)
    if "uniform_random" in new:
        p, parts, _, _ = rt.udf_read(path)
        x = abi.particles_to_numpy(parts, 4)["x"]
        assert np.all((x >= 0) & (x < 32))
        return
    L = rt.load_library()
    p = abi.Params()
    err = C.create_string_buffer(256)
    n = C.c_int()
    st = L.icep_udf_read(os.fsencode(path), C.byref(p), None, 0, C.byref(n), None, None, err, 256)
    assert st == 3, err.value  # ICEP_ERR_UNSUPPORTED
    assert err.value


def test_malformed_and_short_buffer(rt, tmp_path):
    L = rt.load_library()
    p = abi.Params()
    err = C.create_string_buffer(256)
    n = C.c_int()
    bad = rewrite(tmp_path, "A:4.0\n", "A:{4.0\n")  # unbalanced record
    assert L.icep_udf_read(os.fsencode(bad), C.byref(p), None, 0, C.byref(n), None, None, err, 256) == 1
    bad2 = rewrite(tmp_path, '"12:6"', '"13:6"')  # not one of the select's choices
    assert L.icep_udf_read(os.fsencode(bad2), C.byref(p), None, 0, C.byref(n), None, None, err, 256) == 1
    assert b"choices" in err.value
    missing = str(tmp_path / "none.udf")
    assert L.icep_udf_read(os.fsencode(missing), C.byref(p), None, 0, C.byref(n), None, None, err, 256) == 1
    parts = (abi.Particle * 2)()
    assert L.icep_udf_read(os.fsencode(FIX), C.byref(p), parts, 2, C.byref(n), None, None, err, 256) == 1


@pytest.mark.skipif(not os.path.exists(REF_UDF), reason="reference tree not present")
def test_reference_input_udf(rt):
    p, parts, gts, nsnap = rt.udf_read(REF_UDF)
    assert (p.nx, p.ny, p.nz, p.sw_eq) == (32, 32, 32, abi.NAVIER_STOKES)
    assert (gts, nsnap, p.n_particles, p.n_species) == (10, 100, 10, 2)
    assert list(p.mass_ratio)[:2] == [1.5, 0.5]
    assert (p.a, p.a_xi, p.lj_powers, p.g, p.g_direction, p.fix_cell) == (5.0, 2.0, 2, 1.0, 1, 7)
    # auto time step: factor / (nu * KMAX2), KMAX2 = 3 (2 pi / 32 * 11)^2
    kmax2 = 3 * (2 * np.pi / 32 * 11) ** 2
    assert abs(p.dt - 1.0 / kmax2) < 1e-15
    libc = C.CDLL("libc.so.6")
    libc.srand(10)
    r = [libc.rand() / 2147483647 * 32 for _ in range(3)]
    x = abi.particles_to_numpy(parts, 10)["x"]
    assert np.array_equal(x[0], r)
    # the rest of the file binds too (values the path does not use)
    assert rt.udf_value(REF_UDF, "output.ON.EXTENDED.Print_field.YES.Slab_z.stride") == "4"


def test_surface_charges(rt, tmp_path):
    """Charged species are read into surface_charge; mixing charged and
    uncharged species is refused (ICEP_ERR_ARG), as the reference exits."""
    both = rewrite(tmp_path, '{2,1.0,0.0,"Z","OFF"', '{2,1.0,-5.0,"Z","OFF"')
    both2 = open(both).read().replace('{2,1.0,0.0,"X","OFF"', '{2,1.0,3.0,"X","OFF"')
    open(both, "w").write(both2)
    p, _, _, _ = rt.udf_read(both)
    assert list(p.surface_charge)[:2] == [-5.0, 3.0]
    one = rewrite(tmp_path, '{2,1.0,0.0,"Z","OFF"', '{2,1.0,-5.0,"Z","OFF"')
    L = rt.load_library()
    err = C.create_string_buffer(256)
    n = C.c_int()
    st = L.icep_udf_read(os.fsencode(one), C.byref(abi.Params()), None, 0, C.byref(n), None, None, err, 256)
    assert st == 1 and b"Surface_charge" in err.value
