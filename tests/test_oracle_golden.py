"""The C restatement (oracle/icep_oracle.c) against the golden fixtures that
tests/golden/make_golden.py produced by running the reference's own sources."""
import json
import os

import numpy as np
import pytest

import cases
import pyoracle
from icep_kapsel_gb300 import abi

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    with open(os.path.join(GOLD, name + ".json")) as fh:
        meta = json.load(fh)
    return d, meta


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0)


def small_case():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def test_fft16(oracle_so):
    g, _ = load("fft16")
    mg = small_case()
    p, parts = mg.small_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    a = np.random.default_rng(11).standard_normal((16, 16, 18))
    assert rel(o.fft_r2c(a), g["r2c"]) < 1e-14
    # a non-Hermitian spectrum: the reference's C2R reads half of the kz=0
    # and kz=NZ/2 planes (its rdft3dsort packing)
    assert rel(o.fft_c2r(a)[:, :, :16], g["c2r"]) < 1e-14


def test_ops16(oracle_so):
    g, meta = load("ops16")
    mg = small_case()
    p, parts = mg.small_case(potential_tol=mg.OPS16_TOL)
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    f = mg.ops16_inputs(p)
    tol = 1e-12
    o.set("zeta0", f["zeta0"]); o.set("zeta1", f["zeta1"]); o.set_uk_dc(f["uk_dc"])
    o.call("zeta_k2u_k")
    for d in range(3):
        assert rel(o.get("u%d" % d), g["zeta_k2u_k_u%d" % d]) < tol
    o.call("u_k2zeta_k")
    assert rel(o.get("zeta0"), g["u_k2zeta_k_zeta0"]) < tol
    assert rel(o.get("zeta1"), g["u_k2zeta_k_zeta1"]) < tol
    assert rel(o.uk_dc(), g["u_k2zeta_k_ukdc"]) < tol
    for d in range(3):
        o.set("u%d" % d, f["u%d" % d])
    o.call("u2advection_k")
    assert rel(o.get("ns0_0"), g["adv0"]) < tol
    assert rel(o.get("ns0_1"), g["adv1"]) < tol
    for d in range(3):
        o.set("u%d" % d, f["u%d" % d])
    o.call("solenoidal_u")
    for d in range(3):
        assert rel(o.get("u%d" % d)[:, :, :16], g["sol_u%d" % d]) < tol
    o.call("make_phi_sum")
    assert rel(o.get("phi")[:, :, :16], g["phi"]) < tol
    assert rel(o.get("phi_sum")[:, :, :16], g["phi_sum"]) < tol
    o.call("make_u_sum")
    for d in range(3):
        assert rel(o.get("up%d" % d)[:, :, :16], g["up%d" % d]) < tol
    for d in range(3):
        o.set("u%d" % d, f["u%d" % d])
    o.call("f_hydro")
    pa = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["f_hydro"], g["f_hydro"]) < tol
    assert rel(pa["torque_hydro"], g["torque_hydro"]) < tol
    o.call("surface_normal")
    for d in range(3):
        assert rel(o.get("sn%d" % d)[:, :, :16], g["sn%d" % d]) < tol
    o.call("dielectric_field")
    assert rel(o.get("eps")[:, :, :16], g["eps"]) < tol
    assert rel(o.get("work")[:, :, :16], g["phi_sin"]) < tol
    o.call("init_ion")
    assert rel(o.get("c0"), g["c0_init"]) < tol
    assert rel(o.get("c1"), g["c1_init"]) < tol
    o.set("c0", f["c0"]); o.set("c1", f["c1"])
    o.call("charge_field")
    assert rel(o.get("rho")[:, :, :16], g["rho"]) < tol
    o.set("rho", f["rho"])
    o.call("build_rhs")
    assert rel(o.get("work")[:, :, :16], g["rhs"]) < tol
    # Krylov results agree to the solver tolerance (1e-13 here); the
    # potential is defined up to a constant
    o.set("rho", f["rho"]); o.set("pot", f["pot"])
    o.call("solve_potential")
    a = o.get("pot")[:, :, :16]
    b = g["pot_solved"]
    assert rel(a - a.mean(), b - b.mean()) < 1e-11
    assert abs(o.last_iterations() - meta["solve_iterations"]) <= 0.2 * meta["solve_iterations"] + 5
    o.set("rho", f["rho"]); o.set("pot", f["pot"])
    o.set("c0", f["c0"]); o.set("c1", f["c0"])
    o.call("maxwell")
    for d in range(3):
        assert rel(o.get("f%d" % d)[:, :, :16], g["maxwell_f%d" % d]) < tol
    o.set("zeta0", f["zeta0"]); o.set("zeta1", f["zeta1"]); o.set_uk_dc(f["uk_dc"])
    o.set("c0", f["c0"]); o.set("c1", f["c1"]); o.set("pot", f["pot"])
    o.call("nssolute_euler")
    assert rel(o.get("zeta0"), g["np_zeta0"]) < tol
    assert rel(o.get("zeta1"), g["np_zeta1"]) < tol
    assert rel(o.get("c0"), g["np_c0"]) < tol
    assert rel(o.get("c1"), g["np_c1"]) < tol
    o.set("zeta0", f["zeta0"]); o.set("zeta1", f["zeta1"]); o.set_uk_dc(f["uk_dc"])
    o.call("ns_slaved_euler")
    assert rel(o.get("zeta0"), g["ns_zeta0"]) < tol
    assert rel(o.get("zeta1"), g["ns_zeta1"]) < tol


def test_ns32_three_steps(oracle_so):
    g, _ = load("ns32")
    p, parts = cases.ns_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    o.step(3)
    assert rel(o.get("zeta0"), g["zeta0"]) < 1e-12
    assert rel(o.get("zeta1"), g["zeta1"]) < 1e-12
    assert rel(o.get("phi")[:, :, :32], g["phi"]) < 1e-13
    assert rel(o.uk_dc(), g["uk_dc"]) < 1e-12
    pa = abi.particles_to_numpy(o.particles(), p.n_particles)
    for k in ("x", "v", "omega", "q", "f_hydro_previous", "fr_previous"):
        assert rel(pa[k], g["p_" + k]) < 1e-11, k


def test_icep32_two_steps(oracle_so):
    """The reference's step with the spectral solve in its solver seam, to
    1e-12: the restatement follows the same iterates, so every field agrees
    at rounding level."""
    g, meta = load("icep32")
    p, parts = cases.icep_case(tol=1e-12, solver=abi.SOLVER_SPECTRAL)
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    o.step(2)
    for k in ("zeta0", "zeta1", "c0", "c1"):
        assert rel(o.get(k), g[k]) < 1e-12, k
    a = o.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 1e-12
    assert rel(o.get("eps")[:, :, :32], g["eps"]) < 1e-13
    pa = abi.particles_to_numpy(o.particles(), p.n_particles)
    for k in ("x", "v", "omega", "f_hydro_previous", "fr_previous"):
        assert rel(pa[k], g["p_" + k]) < 1e-12, k


def test_icep32_bicgstab_two_steps(oracle_so):
    """The reference's own identity-preconditioned BiCGSTAB (1e-7)."""
    g, meta = load("icep32_bicgstab")
    p, parts = cases.icep_case(tol=1e-7)
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    o.step(2)
    # differences are set by the Poisson tolerance (1e-7): BiCGSTAB iterates
    # of two FFT implementations drift apart at rounding level
    for k in ("zeta0", "zeta1"):
        assert rel(o.get(k), g[k]) < 2e-5, k
    for k in ("c0", "c1"):
        assert rel(o.get(k), g[k]) < 1e-9, k
    a = o.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    assert rel(o.get("eps")[:, :, :32], g["eps"]) < 1e-13
    pa = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["x"], g["p_x"]) < 1e-12
    assert rel(pa["v"], g["p_v"]) < 2e-5


def test_lj32_cell_list_multiplicity(oracle_so):
    g, _ = load("lj32")
    p, parts = cases.lj_dense_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.call("lj")
    fr = abi.particles_to_numpy(o.particles(), p.n_particles)["fr"]
    assert np.abs(fr).max() > 0
    assert rel(fr, g["fr"]) < 1e-13


def test_ax32(oracle_so):
    g, _ = load("ax32")
    p, parts = cases.icep_case(eps_f=1.0, eps_p=10.0)
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.call("dielectric_field")
    x = np.random.default_rng(31).standard_normal(32 * 32 * 32)
    assert rel(o.apply_A(x), g["ax"]) < 1e-13


def test_janus32(oracle_so):
    """Janus dielectric particles (two species, Janus axes z and x, random
    orientations): the permittivity field and two ICEP steps."""
    g, _ = load("janus32")
    p, parts = cases.janus_case(npart=6, axes=(abi.JANUS_Z, abi.JANUS_X), eps_f=4.0, tol=1e-7)
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.call("dielectric_field")
    assert rel(o.get("eps")[:, :, :32], g["eps_field"]) < 1e-13
    assert rel(o.get("work")[:, :, :32], g["phi_p"]) < 1e-13
    # the tanh cap really splits the particles: both eps_top and eps_bottom regions occur
    e = g["eps_field"]
    assert e.max() > 9.0 and e.min() < 2.5
    o.init_state()
    o.step(2)
    for k in ("zeta0", "zeta1"):
        assert rel(o.get(k), g[k]) < 2e-5, k
    for k in ("c0", "c1"):
        assert rel(o.get(k), g[k]) < 1e-9, k
    a = o.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    assert rel(o.get("eps")[:, :, :32], g["eps"]) < 1e-13
    pa = abi.particles_to_numpy(o.particles(), p.n_particles)
    assert rel(pa["x"], g["p_x"]) < 1e-12


def test_charged32(oracle_so):
    """Charged particles (Init_rho_ion's counterions, Conc_k2charge_field with
    Make_phi_qq_particle) and the initial potential."""
    g, meta = load("charged32")
    p, parts = cases.charged_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    for k in ("c0", "c1"):
        assert rel(o.get(k), g[k]) < 1e-14, k
    a = o.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    o.call("charge_field")
    assert rel(o.get("rho")[:, :, :32], g["rho"]) < 1e-13
    assert rel(o.get("work")[:, :, :32], g["phi_p"]) < 1e-13
    # the surface term is there: the charge field is far from the salt-only one
    assert np.abs(g["rho"]).max() > 1e-3


def test_ac32(oracle_so):
    """An AC external field (E_ext sin(2 pi f t)): the field is zero at t = 0,
    so the initial solve and the first step's give a zero potential, and the
    next two steps solve, move ions and drive the fluid with the field at
    t = dt and 2 dt."""
    g, meta = load("ac32")
    p, parts = cases.ac_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    o.step(1)
    assert meta["step0_iterations"] == 0 and np.abs(g["pot_step0"]).max() == 0.0
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
    # the phase matters: the same steps under the DC field differ at first order
    q, qparts = cases.ac_case()
    q.ac = 0
    d = pyoracle.Oracle(q, qparts, so=oracle_so)
    d.init_state()
    d.step(3)
    b = d.get("pot")[:, :, :32]
    assert rel(b - b.mean(), g["pot"] - g["pot"].mean()) > 0.05


def test_out32(oracle_so):
    """The fields of the field output (Output_dielectric_charge_field_data,
    restated in the reference harness around its own Zeta_k2u and
    Make_phi_qq_particle): u with a mean flow, the unclipped phi, the
    surface charge times 4 pi a^2, the solute charge and eps; with uncharged
    particles the surface charge is 0/0 = NaN in the reference and here."""
    g, meta = load("out32")
    ic, _ = load("icep32_bicgstab")
    p, parts = cases.charged_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    o.set("zeta0", ic["zeta0"])
    o.set("zeta1", ic["zeta1"])
    o.set_uk_dc(np.array([30.0, -60.0, 15.0]))
    o.call("charge_output")
    for k in ("u0", "u1", "u2"):
        assert rel(o.get(k)[:, :, :32], g[k]) < 1e-13, k
    assert abs(g["u0"].mean() - 30.0 / 32 ** 3) < 1e-15
    assert rel(o.get("phi")[:, :, :32], g["phi"]) < 1e-14
    assert rel(o.get("up0")[:, :, :32], g["up0"]) < 1e-13
    assert rel(o.get("up1")[:, :, :32], g["up1"]) < 1e-12
    assert rel(o.get("up2")[:, :, :32], g["up2"]) < 1e-13
    assert meta["uncharged_surface_all_nan"]
    q, qparts = cases.icep_case()
    t = pyoracle.Oracle(q, qparts, so=oracle_so)
    t.init_state()
    t.call("charge_output")
    assert np.all(np.isnan(t.get("up0")[:, :, :32]))


def test_saltfree32(oracle_so):
    """Salt-free electrolyte (Add_salt saltfree, N_spec = 1): the counterions
    of two negatively charged species spread evenly over the fluid volume
    (Init_rho_ion with Set_uniform_ion_charge_density_nosalt), the charge
    field and the initial potential; the absent second species stays zero."""
    g, meta = load("saltfree32")
    p, parts = cases.saltfree_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    assert rel(o.get("c0"), g["c0"]) < 1e-14
    assert np.abs(o.get("c1")).max() == 0.0
    # 16 counterions (charges -5, -3 on two particles each) over the fluid volume
    assert abs(g["c0"][0, 0, 0] / 32 ** 3 * (32 ** 3 - 4 * 268.0) - 16.0) < 0.5
    a = o.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
    o.call("charge_field")
    assert rel(o.get("rho")[:, :, :32], g["rho"]) < 1e-12


def test_charged32_pb(oracle_so):
    """INIT_profile Poisson_Boltzmann (Set_steadystate_ion_density): the
    relaxed ion densities at rounding level -- the relaxation stops at the same
    step (its free-energy test) and every step agrees."""
    g, meta = load("charged32_pb")
    p, parts = cases.pb_case()
    o = pyoracle.Oracle(p, parts, so=oracle_so)
    o.init_state()
    assert o.pb_iterations() > 10
    for k in ("c0", "c1"):
        assert rel(o.get(k), g[k]) < 1e-12, k
    a = o.get("pot")[:, :, :32]
    assert rel(a - a.mean(), g["pot"] - g["pot"].mean()) < 2e-5
