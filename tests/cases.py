"""Seeded test and benchmark cases (shared by tests, fixture generation and bench).

Synthetic inputs only: particle centres are drawn from numpy's PCG64 generator
with a minimum periodic separation; the fluid starts at rest.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from icep_kapsel_gb300 import abi  # noqa: E402


def positions(n, L, minsep, seed, max_tries=200000):
    """n centres uniform in [0,L)^3 with periodic separation >= minsep."""
    rng = np.random.default_rng(seed)
    L = np.asarray(L, dtype=np.float64) * np.ones(3)
    out = []
    tries = 0
    while len(out) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("cannot place %d particles with separation %g" % (n, minsep))
        x = rng.uniform(0.0, 1.0, 3) * L
        ok = True
        for y in out:
            d = x - y
            d -= L * np.round(d / L)
            if np.dot(d, d) < minsep * minsep:
                ok = False
                break
        if ok:
            out.append(x)
    return np.array(out).reshape(n, 3)


def ns_case(n=32, npart=8, minsep=10.0, seed=1, rotation=1, dt=0.05, motor=True):
    """Plain SPM DNS: n^3, dx=1, rho=eta=1, spheres a=4 xi=2, WCA 12:6,
    particle 0 pushed by a body-frame force 0.01 along x (a motor species;
    the reference requires ROTATION ON for motor particles)."""
    x = positions(npart, n, minsep, seed)
    spec = [0] + [1] * (npart - 1) if motor else [0] * npart
    p = abi.make_params(nx=n, ny=n, nz=n, n_particles=npart, n_species=2 if motor else 1,
                        rotation=rotation, dt=dt, a=4.0, a_xi=2.0, lj_epsilon=1.0, lj_powers=0,
                        lj_truncate=1,
                        janus_propulsion=[abi.MOTOR, abi.NO_PROPULSION] if motor else [abi.NO_PROPULSION],
                        janus_force=[[0.01, 0.0, 0.0], [0.0, 0.0, 0.0]])
    return p, abi.make_particles(x, spec=spec)


def icep_case(n=32, npart=4, minsep=12.0, seed=2, a=4.0, eps_f=1.0, eps_p=10.0, e_ext=(0.01, 0.0, 0.0),
              tol=1e-6, maxit=2000, dt=0.01, per_particle_eps=None, solver=abi.SOLVER_REF,
              precision=abi.FP64):
    """Electrolyte + Dielectric_property ON, salt (z=+-1, Onsager 7.24,
    Debye length 10 a), kBT=1, Dielectric_cst=1 (the reference's sample
    input values), uniform external field."""
    x = positions(npart, n, minsep, seed)
    eps = None
    if per_particle_eps is not None:
        lo, hi = per_particle_eps
        eps = np.random.default_rng(seed + 1000).uniform(lo, hi, npart)
    p = abi.make_params(nx=n, ny=n, nz=n, n_particles=npart, n_species=1, sw_eq=abi.ELECTROLYTE,
                        dielectric=1, dielectric_cst=1.0, eps_fluid=eps_f, eps_particle_top=eps_p,
                        eps_particle_bottom=eps_p, external_field=1, e_ext=list(e_ext),
                        potential_tol=tol, potential_iter=maxit, kbt=1.0, debye_length=10.0,
                        onsager_pos=7.24, onsager_neg=7.24, valency_pos=1.0, valency_neg=-1.0,
                        dt=dt, a=a, a_xi=2.0, rotation=0, per_particle_eps=1 if eps is not None else 0,
                        solver=solver, precision=precision)
    return p, abi.make_particles(x, eps_p=eps)


def ac_case(frequency=8.0, tol=1e-7, solver=abi.SOLVER_REF, precision=abi.FP64):
    """An AC external field E_ext sin(2 pi f t) (Electric_field.ON.AC): with
    dt = 0.01 and f = 8 the phase advances 0.5 rad a step, so the field is
    zero at t = 0 (the initial solve and the first step) and grows after."""
    p, parts = icep_case(e_ext=(0.0, 0.05, 0.1), tol=tol, solver=solver, precision=precision)
    p.ac = 1
    p.frequency = frequency
    return p, parts


def splitmix64(n, seed):
    """n pseudo-random uint64 (splitmix64), reproducible on any numpy."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def avs_inputs(nx, ny, nz, npart, seed=7):
    """Inputs for the AVS writers: 7 fields in the [NX][NY][NZ_] layout with
    values of ~40 significant bits (so the float32 cast rounds) and signs,
    particle positions in the box and unit quaternions."""
    nz_ = 2 * (nz // 2 + 1)
    n = nx * ny * nz_
    fields = []
    for v in range(7):
        r = splitmix64(n, seed + v).astype(np.float64) / 2.0 ** 64  # [0, 1)
        fields.append(np.ascontiguousarray(((r - 0.5) * 10.0 ** (v - 3)).reshape(nx, ny, nz_)))
    r = splitmix64(npart * 7, seed + 100).astype(np.float64) / 2.0 ** 64
    x = r[:3 * npart].reshape(npart, 3) * np.array([nx, ny, nz], dtype=np.float64)
    q = r[3 * npart:].reshape(npart, 4) - 0.5
    q = q / np.sqrt((q * q).sum(axis=1, keepdims=True))
    return fields, x, q


def unit_quaternions(n, seed):
    """n orientations uniform on the rotation group (normalised Gaussian 4-vectors)."""
    q = np.random.default_rng(seed).standard_normal((n, 4))
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def janus_case(n=32, npart=4, minsep=12.0, seed=4, axes=(abi.JANUS_Z,), eps_top=10.0, eps_bottom=2.0,
               eps_f=80.0, e_ext=(0.0, 0.0, 0.1), tol=1e-8, maxit=2000, solver=abi.SOLVER_REF,
               precision=abi.FP64):
    """Janus dielectric particles (Make_janus_permittivity_dielectric): one
    species per entry of `axes` (particles assigned round-robin), the cap
    eps_top on the +e3 side and eps_bottom on the other, random orientations."""
    p, _ = icep_case(n=n, npart=npart, minsep=minsep, seed=seed, eps_f=eps_f, eps_p=eps_top, e_ext=e_ext,
                     tol=tol, maxit=maxit, solver=solver, precision=precision)
    p.n_species = len(axes)
    for i, a in enumerate(axes):
        p.janus_axis[i] = a
        p.mass_ratio[i] = 1.0
    p.eps_particle_bottom = eps_bottom
    x = positions(npart, n, minsep, seed)
    spec = [i % len(axes) for i in range(npart)]
    return p, abi.make_particles(x, spec=spec, q=unit_quaternions(npart, seed + 500))


def charged_case(n=32, npart=4, seed=2, charges=(-5.0,), tol=1e-7, solver=abi.SOLVER_REF, precision=abi.FP64,
                 eps_f=1.0, eps_p=10.0, e_ext=(0.01, 0.0, 0.0)):
    """Charged particles in the salt solution (Init_rho_ion +
    Conc_k2charge_field with Make_phi_qq_particle): one species per entry of
    `charges` (particles assigned round-robin)."""
    p, _ = icep_case(n=n, npart=npart, seed=seed, eps_f=eps_f, eps_p=eps_p, e_ext=e_ext, tol=tol, solver=solver,
                     precision=precision)
    p.n_species = len(charges)
    for i, q in enumerate(charges):
        p.surface_charge[i] = q
        p.mass_ratio[i] = 1.0
    x = positions(npart, n, 12.0, seed)
    return p, abi.make_particles(x, spec=[i % len(charges) for i in range(npart)])


def pb_case(precision=abi.FP64, solver=abi.SOLVER_REF, tol=1e-7):
    """Charged particles in the salt solution with INIT_profile
    Poisson_Boltzmann and a DC field E0 = (0, 0, 0.1): the ion densities are
    relaxed towards their steady state in the field before the first solve."""
    p, parts = charged_case(e_ext=(0.0, 0.0, 0.1), precision=precision, solver=solver, tol=tol)
    p.poisson_boltzmann = 1
    return p, parts


def saltfree_case(n=32, npart=4, seed=2, charges=(-5.0, -3.0), tol=1e-7, solver=abi.SOLVER_REF,
                  precision=abi.FP64, valency=1.0, onsager=7.24):
    """Charged particles with their counterions only (Add_salt saltfree,
    N_spec = 1): two negatively charged species, monovalent counterions;
    the salt keys are zeroed to show they are not used."""
    p, parts = charged_case(n=n, npart=npart, seed=seed, charges=charges, tol=tol, solver=solver,
                            precision=precision)
    p.salt_free = 1
    p.valency_counterion = valency
    p.onsager_counterion = onsager
    p.valency_pos = p.valency_neg = 0.0
    p.onsager_pos = p.onsager_neg = 0.0
    p.debye_length = 0.0
    return p, parts


def lj_dense_case(n=32, npart=24, seed=7, minsep=7.2):
    """Particles closer than the WCA cutoff (2^(1/6) * 8 = 8.98) so that the
    cell-list scan and its multiplicity at 32^3 (2 cells per side) matter."""
    x = positions(npart, n, minsep, seed)
    p = abi.make_params(nx=n, ny=n, nz=n, n_particles=npart, n_species=1, rotation=0, dt=0.05)
    return p, abi.make_particles(x)


def icep64_case(solver=abi.SOLVER_SPECTRAL, precision=abi.FP64, tol=1e-10):
    """The plain ICEP run at 64^3: 16 dielectric spheres a = 5, xi = 2,
    eps_particle = 2, eps_fluid = 80, centres uniform-random with minimum
    separation 12, uniform external field E0 = (0, 0, 0.1), Poisson solved to
    1e-10 true residual (the salt of icep_case)."""
    return icep_case(n=64, npart=16, minsep=12.0, seed=64, a=5.0, eps_f=80.0, eps_p=2.0,
                     e_ext=(0.0, 0.0, 0.1), tol=tol, solver=solver, precision=precision)


def _rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0))


def mixed_vs_oracle_errors(m, o, nz, npart):
    """Relative L2 error per field of a MIXED GPU state against the FP64
    oracle's state (velocity from the vorticity by Zeta_k2u on both sides)."""
    out = {}
    for k in ("zeta0", "zeta1", "c0", "c1"):
        out[k] = _rel(m.get(k), o.get(k))
    a, b = m.get("pot")[:, :, :nz], o.get("pot")[:, :, :nz]
    out["pot"] = _rel(a - a.mean(), b - b.mean())
    out["phi"] = _rel(m.get("phi")[:, :, :nz], o.get("phi")[:, :, :nz])
    m.call("zeta_k2u")
    o.call("zeta_k2u")
    out["u"] = float(np.sqrt(sum(np.linalg.norm(m.get("u%d" % d)[:, :, :nz] - o.get("u%d" % d)[:, :, :nz]) ** 2
                                 for d in range(3)) /
                             sum(np.linalg.norm(o.get("u%d" % d)[:, :, :nz]) ** 2 for d in range(3))))
    pa = abi.particles_to_numpy(m.particles(), npart)
    pb = abi.particles_to_numpy(o.particles(), npart)
    for k in ("x", "v"):
        out["particle_" + k] = _rel(pa[k], pb[k])
    return out
