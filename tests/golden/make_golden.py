"""Generate the golden fixtures in this directory from the reference's own code.

Runs the reference's hot-path sources compiled by oracle/ref/Makefile
(oracle/_ref/libkapsel_ref.so: Ooura FFT, fft_wrapper, operate_omega,
fluid_solver, make_phi, md_force, particle_solver, operate_dielectric,
solute_rhs, operate_electrolyte, plus the restated BiCGSTAB behind the Eigen
shim) on the seeded cases of tests/cases.py and stores the outputs.

Needs the reference tree (--ref, else oracle/pyoracle.py ref_dir()); the fixtures it writes are
committed so that the tests run without it:

    python tests/golden/make_golden.py [--ref <reference source tree>]

Each case runs in its own process because the reference keeps its state in
process globals.
"""
import argparse
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CASES = ["fft16", "ops16", "ns32", "icep32", "icep32_bicgstab", "icep64_200", "lj32", "ax32", "janus32", "charged32", "charged32_pb", "ac32", "out32", "avs16", "saltfree32"]


def small_case(potential_tol=1e-10):
    """16^3 with a=2 spheres (stencil radius 4.7 < 8) for operator fixtures.
    The ops16 fixture solves to 1e-13 so that everything downstream of its
    Poisson solves (the potential, the Maxwell force) is pinned at 1e-12."""
    import cases
    from icep_kapsel_gb300 import abi
    x = cases.positions(3, 16, 6.0, 21)
    p = abi.make_params(nx=16, ny=16, nz=16, n_particles=3, n_species=1, a=2.0, a_xi=2.0,
                        rotation=1, dt=0.05, sw_eq=abi.ELECTROLYTE, dielectric=1,
                        eps_fluid=1.0, eps_particle_top=10.0, eps_particle_bottom=10.0,
                        external_field=1, e_ext=[0.01, 0.002, -0.003], potential_tol=potential_tol,
                        potential_iter=3000, kbt=1.0, debye_length=10.0, onsager_pos=7.24,
                        onsager_neg=7.24)
    rng = np.random.default_rng(99)
    v = rng.uniform(-0.05, 0.05, (3, 3))
    parts = abi.make_particles(x, v=v)
    for i in range(3):
        for d in range(3):
            parts[i].omega[d] = rng.uniform(-0.01, 0.01)
    return p, parts


OPS16_TOL = 1e-13
ICEP64_STEPS = 200


def ops16_inputs(p):
    """Seeded random fields for the isolated-operator fixture."""
    rng = np.random.default_rng(1234)
    shp = (p.nx, p.ny, 2 * (p.nz // 2 + 1))
    f = {}
    for k in ("zeta0", "zeta1", "u0", "u1", "u2"):
        f[k] = rng.standard_normal(shp) * 0.01
        if k.startswith("u"):
            f[k][:, :, p.nz:] = 0.0
    f["uk_dc"] = rng.standard_normal(3) * 0.01
    f["c0"] = rng.standard_normal(shp) * 1e-3
    f["c1"] = rng.standard_normal(shp) * 1e-3
    f["pot"] = rng.standard_normal(shp) * 0.1
    f["pot"][:, :, p.nz:] = 0.0
    f["rho"] = rng.standard_normal(shp) * 1e-4
    f["rho"][:, :, p.nz:] = 0.0
    # a charge-neutral density keeps the singular Poisson system consistent
    f["rho"][:, :, :p.nz] -= f["rho"][:, :, :p.nz].mean()
    return f


def run_case(name, out):
    import cases
    import pyoracle
    from icep_kapsel_gb300 import abi
    meta = {"case": name}
    data = {}
    if name == "fft16":
        p, parts = small_case()
        r = pyoracle.RefKapsel(p, parts)
        a = np.random.default_rng(11).standard_normal((16, 16, 18))
        data["r2c"] = r.fft_r2c(a)
        data["c2r"] = r.fft_c2r(a)[:, :, :16]
    elif name == "ops16":
        p, parts = small_case(potential_tol=OPS16_TOL)
        r = pyoracle.RefKapsel(p, parts)
        f = ops16_inputs(p)
        # Zeta_k2u_k
        r.set("zeta0", f["zeta0"]); r.set("zeta1", f["zeta1"]); r.set_uk_dc(f["uk_dc"])
        r.call("zeta_k2u_k")
        for d in range(3):
            data["zeta_k2u_k_u%d" % d] = r.get("u%d" % d)
        # U_k2zeta_k on the same u
        r.call("u_k2zeta_k")
        data["u_k2zeta_k_zeta0"] = r.get("zeta0"); data["u_k2zeta_k_zeta1"] = r.get("zeta1")
        data["u_k2zeta_k_ukdc"] = r.uk_dc()
        # U2advection_k from a real field
        for d in range(3):
            r.set("u%d" % d, f["u%d" % d])
        r.call("u2advection_k")
        data["adv0"] = r.get("ns0_0"); data["adv1"] = r.get("ns0_1")
        # Solenoidal_u
        for d in range(3):
            r.set("u%d" % d, f["u%d" % d])
        r.call("solenoidal_u")
        for d in range(3):
            data["sol_u%d" % d] = r.get("u%d" % d)[:, :, :16]
        # profile scatters and gathers
        r.call("make_phi_sum")
        data["phi"] = r.get("phi")[:, :, :16]; data["phi_sum"] = r.get("phi_sum")[:, :, :16]
        r.call("make_u_sum")
        for d in range(3):
            data["up%d" % d] = r.get("up%d" % d)[:, :, :16]
        for d in range(3):
            r.set("u%d" % d, f["u%d" % d])
        r.call("f_hydro")
        pa = abi.particles_to_numpy(r.particles(), p.n_particles)
        data["f_hydro"] = pa["f_hydro"]; data["torque_hydro"] = pa["torque_hydro"]
        r.call("surface_normal")
        for d in range(3):
            data["sn%d" % d] = r.get("sn%d" % d)[:, :, :16]
        # dielectric pieces
        r.call("dielectric_field")
        data["eps"] = r.get("eps")[:, :, :16]
        data["phi_sin"] = r.get("work")[:, :, :16]
        r.set("c0", f["c0"]); r.set("c1", f["c1"])
        r.call("init_ion")
        data["c0_init"] = r.get("c0"); data["c1_init"] = r.get("c1")
        r.set("c0", f["c0"]); r.set("c1", f["c1"])
        r.call("charge_field")
        data["rho"] = r.get("rho")[:, :, :16]
        r.set("rho", f["rho"])
        r.call("build_rhs")
        data["rhs"] = r.get("work")[:, :, :16]
        r.set("rho", f["rho"]); r.set("pot", f["pot"])
        r.call("solve_potential")
        data["pot_solved"] = r.get("pot")[:, :, :16]
        meta["solve_iterations"] = int(r.last_iterations())
        meta["solve_error"] = float(r.last_error())
        # equal salt concentrations: zero free charge, a consistent solve
        r.set("rho", f["rho"]); r.set("pot", f["pot"])
        r.set("c0", f["c0"]); r.set("c1", f["c0"])
        r.call("maxwell")
        meta["maxwell_iterations"] = int(r.last_iterations())
        for d in range(3):
            data["maxwell_f%d" % d] = r.get("f%d" % d)[:, :, :16]
        data["maxwell_pot"] = r.get("pot")[:, :, :16]
        # NSsolute_solver_Euler
        r.set("zeta0", f["zeta0"]); r.set("zeta1", f["zeta1"]); r.set_uk_dc(f["uk_dc"])
        r.set("c0", f["c0"]); r.set("c1", f["c1"]); r.set("pot", f["pot"])
        r.call("nssolute_euler")
        data["np_zeta0"] = r.get("zeta0"); data["np_zeta1"] = r.get("zeta1")
        data["np_c0"] = r.get("c0"); data["np_c1"] = r.get("c1")
        # NS_solver_slavedEuler
        r.set("zeta0", f["zeta0"]); r.set("zeta1", f["zeta1"]); r.set_uk_dc(f["uk_dc"])
        r.call("ns_slaved_euler")
        data["ns_zeta0"] = r.get("zeta0"); data["ns_zeta1"] = r.get("zeta1")
    elif name == "ns32":
        p, parts = cases.ns_case()
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        r.step(3)
        data["zeta0"] = r.get("zeta0"); data["zeta1"] = r.get("zeta1")
        data["phi"] = r.get("phi")[:, :, :32]
        data["uk_dc"] = r.uk_dc()
        for k, v in abi.particles_to_numpy(r.particles(), p.n_particles).items():
            data["p_" + k] = v
    elif name in ("icep32", "icep32_bicgstab"):
        # icep32: the reference's step with the plain spectral solve of the
        # GPU path installed in its solver seam, to 1e-12 (fields pinned at
        # 1e-10); icep32_bicgstab: the reference's own identity-preconditioned
        # BiCGSTAB, which reaches 1e-7 on this case but not 1e-12 (the
        # periodic system turns inconsistent as the ions move)
        if name == "icep32":
            p, parts = cases.icep_case(tol=1e-12, solver=abi.SOLVER_SPECTRAL)
        else:
            p, parts = cases.icep_case(tol=1e-7)
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        meta["init_iterations"] = int(r.last_iterations())
        r.step(2)
        meta["step_iterations"] = int(r.last_iterations())
        meta["step_error"] = float(r.last_error())
        for k in ("zeta0", "zeta1", "c0", "c1"):
            data[k] = r.get(k)
        data["pot"] = r.get("pot")[:, :, :32]
        data["eps"] = r.get("eps")[:, :, :32]
        data["uk_dc"] = r.uk_dc()
        for k, v in abi.particles_to_numpy(r.particles(), p.n_particles).items():
            data["p_" + k] = v
    elif name == "icep64_200":
        # the plain ICEP run at 64^3 (16 dielectric spheres a = 5, eps_p = 2,
        # eps_f = 80, E0 = (0, 0, 0.1), Poisson to 1e-10 true residual) for
        # 200 steps; fields are stored on every 4th point of each axis (the
        # full fields would be 11 MB) with their full-grid norms
        p, parts = cases.icep64_case()
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        its = [int(r.last_iterations())]
        for _ in range(ICEP64_STEPS):
            r.step(1)
            its.append(int(r.last_iterations()))
        meta["iterations"] = its
        meta["step_error"] = float(r.last_error())
        for k in ("zeta0", "zeta1", "c0", "c1"):
            a = r.get(k)
            data[k] = a[::4, ::4, ::4]
            data[k + "_norm"] = np.linalg.norm(a)
        for k in ("pot", "phi"):
            a = r.get(k)[:, :, :64]
            if k == "pot":  # defined up to a constant
                a = a - a.mean()
            data[k] = a[::4, ::4, ::4]
            data[k + "_norm"] = np.linalg.norm(a)
        data["uk_dc"] = r.uk_dc()
        for k, v in abi.particles_to_numpy(r.particles(), p.n_particles).items():
            data["p_" + k] = v
    elif name == "lj32":
        p, parts = cases.lj_dense_case()
        r = pyoracle.RefKapsel(p, parts)
        r.call("lj")
        data["fr"] = abi.particles_to_numpy(r.particles(), p.n_particles)["fr"]
    elif name == "ax32":
        p, parts = cases.icep_case(eps_f=1.0, eps_p=10.0)
        r = pyoracle.RefKapsel(p, parts)
        r.call("dielectric_field")
        x = np.random.default_rng(31).standard_normal(32 * 32 * 32)
        data["ax"] = r.apply_A(x)
    elif name == "janus32":
        # two species with different Janus axes, random orientations; a
        # moderate permittivity contrast so that the reference's
        # unpreconditioned BiCGSTAB converges within its iteration limit
        p, parts = cases.janus_case(npart=6, axes=(abi.JANUS_Z, abi.JANUS_X), eps_f=4.0, tol=1e-7)
        r = pyoracle.RefKapsel(p, parts)
        r.call("dielectric_field")
        data["eps_field"] = r.get("eps")[:, :, :32]
        data["phi_p"] = r.get("work")[:, :, :32]
        r.init_state()
        meta["init_iterations"] = int(r.last_iterations())
        r.step(2)
        meta["step_iterations"] = int(r.last_iterations())
        meta["step_error"] = float(r.last_error())
        for k in ("zeta0", "zeta1", "c0", "c1"):
            data[k] = r.get(k)
        data["pot"] = r.get("pot")[:, :, :32]
        data["eps"] = r.get("eps")[:, :, :32]
        for k, v in abi.particles_to_numpy(r.particles(), p.n_particles).items():
            data["p_" + k] = v
    elif name == "charged32":
        # charged particles: counterion initialisation, the surface-charge
        # field and the initial Poisson solve (the reference's unpreconditioned
        # BiCGSTAB does not reach 1e-7 in the steps after it: the periodic
        # system turns inconsistent as the ions move, so steps are compared
        # with the spectral solver elsewhere)
        p, parts = cases.charged_case()
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        meta["init_iterations"] = int(r.last_iterations())
        meta["init_error"] = float(r.last_error())
        for k in ("c0", "c1"):
            data[k] = r.get(k)
        data["pot"] = r.get("pot")[:, :, :32]
        r.call("charge_field")
        data["rho"] = r.get("rho")[:, :, :32]
        data["phi_p"] = r.get("work")[:, :, :32]
    elif name == "charged32_pb":
        # INIT_profile Poisson_Boltzmann with charged particles in the salt
        # solution: Init_rho_ion relaxes the uniform densities in the external
        # field (Set_steadystate_ion_density) before the initial solve
        p, parts = cases.pb_case()
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        meta["init_iterations"] = int(r.last_iterations())
        meta["init_error"] = float(r.last_error())
        for k in ("c0", "c1"):
            data[k] = r.get(k)
        data["pot"] = r.get("pot")[:, :, :32]
    elif name == "ac32":
        # an AC field: zero at t = 0 (initial solve and first step), then
        # E_ext sin(2 pi f t) in the Poisson right-hand side, the ions' flux
        # and the Maxwell stress of the next two steps
        p, parts = cases.ac_case()
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        meta["init_iterations"] = int(r.last_iterations())
        r.step(1)
        meta["step0_iterations"] = int(r.last_iterations())
        data["pot_step0"] = r.get("pot")[:, :, :32]
        r.step(2)
        meta["step_iterations"] = int(r.last_iterations())
        meta["step_error"] = float(r.last_error())
        for k in ("zeta0", "zeta1", "c0", "c1"):
            data[k] = r.get(k)
        data["pot"] = r.get("pot")[:, :, :32]
        for k, v in abi.particles_to_numpy(r.particles(), p.n_particles).items():
            data["p_" + k] = v
    elif name == "out32":
        # the field output (Output_dielectric_charge_field_data's fields) of
        # the charged case after its initial solve, with a flow: zeta from
        # the icep32 fixture and a mean velocity uk_dc
        ic = np.load(os.path.join(HERE, "icep32_bicgstab.npz"))
        p, parts = cases.charged_case()
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        r.set("zeta0", ic["zeta0"])
        r.set("zeta1", ic["zeta1"])
        r.set_uk_dc(np.array([30.0, -60.0, 15.0]))  # the k = 0 coefficient: N times the mean
        r.call("charge_output")
        for k in ("u0", "u1", "u2", "phi", "up0", "up1", "up2"):
            data[k] = r.get(k)[:, :, :32]
        data["pot"] = r.get("pot")[:, :, :32]
        # uncharged particles: the surface charge's rescale is 0/0
        q, qparts = cases.icep_case()
        t = pyoracle.RefKapsel(q, qparts)
        t.init_state()
        t.call("charge_output")
        meta["uncharged_surface_all_nan"] = bool(np.all(np.isnan(t.get("up0")[:, :, :32])))
    elif name == "avs16":
        # the reference's AVS writers (binary and ASCII) on seeded fields and
        # particles: the SHA-256 of every file they write, and the text of
        # the headers (the scratch directories are removed afterwards)
        import hashlib
        import shutil
        p, _ = small_case()
        fields, x, q = cases.avs_inputs(16, 16, 16, p.n_particles)
        parts = abi.make_particles(x)
        for i in range(p.n_particles):
            for d in range(4):
                parts[i].q[d] = q[i, d]
                parts[i].q_old[d] = q[i, d]
        r = pyoracle.RefKapsel(p, parts)
        r.set_ts(20, 0.25)
        files, text = {}, {}
        for ascii in (0, 1):
            d = os.path.join(HERE, "_avs16_scratch_%d" % ascii)
            shutil.rmtree(d, ignore_errors=True)
            os.makedirs(d)
            r.avs(d, "data", ascii, 5, fields)
            for root, _, names in os.walk(d):
                for nm in names:
                    path = os.path.join(root, nm)
                    rel = "%d/%s" % (ascii, os.path.relpath(path, d))
                    blob = open(path, "rb").read()
                    files[rel] = [hashlib.sha256(blob).hexdigest(), len(blob)]
                    if nm.endswith(".fld") or nm == "data.cod":
                        text[rel] = blob.decode()
            shutil.rmtree(d)
        meta["files"] = files
        meta["text"] = text
    elif name == "saltfree32":
        # counterions only (N_spec = 1): the uniform counterion density over
        # the fluid volume, the charge field and the initial potential
        p, parts = cases.saltfree_case()
        r = pyoracle.RefKapsel(p, parts)
        r.init_state()
        meta["init_iterations"] = int(r.last_iterations())
        meta["init_error"] = float(r.last_error())
        data["c0"] = r.get("c0")
        data["pot"] = r.get("pot")[:, :, :32]
        r.call("charge_field")
        data["rho"] = r.get("rho")[:, :, :32]
    else:
        raise ValueError(name)
    meta["params"] = abi.params_dict(p)
    np.savez_compressed(out, **data)
    with open(out.replace(".npz", ".json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


def main():
    ap = argparse.ArgumentParser()
    import pyoracle
    ap.add_argument("--ref", default=pyoracle.ref_dir())
    ap.add_argument("--case", default=None)
    a = ap.parse_args()
    if a.case:
        run_case(a.case, os.path.join(HERE, a.case + ".npz"))
        return
    import pyoracle
    if not pyoracle.build_ref(a.ref):
        sys.exit("reference tree not found: " + a.ref)
    for c in CASES:
        print("case", c, flush=True)
        subprocess.check_call([sys.executable, __file__, "--case", c, "--ref", a.ref])


if __name__ == "__main__":
    main()
