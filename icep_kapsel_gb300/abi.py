"""ctypes mirrors of include/icep_types.h and parameter helpers.

The field names and meanings follow the reference's input.udf keys and globals
(input.cxx:286-440 derives the remaining quantities); see the header for the
layout conventions of fields and particles.
"""
import ctypes as C

import numpy as np

MAX_SPECIES = 4
NAVIER_STOKES = 0
ELECTROLYTE = 3
MOTOR = 0
NO_PROPULSION = 3
FP64 = 0
MIXED = 1
SOLVER_REF = 0
SOLVER_SPECTRAL = 1
SOLVER_LEARNED = 2
JANUS_NONE, JANUS_X, JANUS_Y, JANUS_Z = 0, 1, 2, 3


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("sw_eq", C.c_int),
        ("dx", C.c_double), ("rho", C.c_double), ("eta", C.c_double), ("kbt", C.c_double),
        ("dt", C.c_double),
        ("a", C.c_double), ("a_xi", C.c_double),
        ("lj_epsilon", C.c_double),
        ("lj_powers", C.c_int),
        ("lj_truncate", C.c_int),
        ("rotation", C.c_int),
        ("fixed_particle", C.c_int),
        ("n_particles", C.c_int),
        ("n_species", C.c_int),
        ("mass_ratio", C.c_double * MAX_SPECIES),
        ("janus_propulsion", C.c_int * MAX_SPECIES),
        ("janus_force", (C.c_double * 3) * MAX_SPECIES),
        ("janus_torque", (C.c_double * 3) * MAX_SPECIES),
        ("g", C.c_double),
        ("g_direction", C.c_int),
        ("dielectric", C.c_int),
        ("dielectric_cst", C.c_double),
        ("eps_fluid", C.c_double),
        ("eps_particle_top", C.c_double),
        ("eps_particle_bottom", C.c_double),
        ("potential_iter", C.c_int),
        ("potential_tol", C.c_double),
        ("valency_pos", C.c_double), ("valency_neg", C.c_double),
        ("onsager_pos", C.c_double), ("onsager_neg", C.c_double),
        ("debye_length", C.c_double),
        ("elementary_charge", C.c_double),
        ("external_field", C.c_int),
        ("e_ext", C.c_double * 3),
        ("precision", C.c_int),
        ("solver", C.c_int),
        ("per_particle_eps", C.c_int),
        ("janus_axis", C.c_int * MAX_SPECIES),
        ("fix_cell", C.c_int),
        ("surface_charge", C.c_double * MAX_SPECIES),
        ("ac", C.c_int),
        ("frequency", C.c_double),
        ("salt_free", C.c_int),
        ("valency_counterion", C.c_double),
        ("onsager_counterion", C.c_double),
        ("poisson_boltzmann", C.c_int),
    ]


class Particle(C.Structure):
    _fields_ = [("spec", C.c_int), ("pad_", C.c_int)] + [
        (n, C.c_double * 3) for n in (
            "x", "x_nopbc", "v", "v_old", "omega", "omega_old",
            "f_hydro", "f_hydro_previous", "f_hydro1", "fr", "fr_previous",
            "torque_hydro", "torque_hydro_previous", "torque_hydro1",
            "torque_r", "torque_r_previous")
    ] + [("q", C.c_double * 4), ("q_old", C.c_double * 4), ("eps_p", C.c_double)]


PARTICLE_VEC_FIELDS = [n for n, _ in Particle._fields_ if n not in ("spec", "pad_", "eps_p")]


def make_params(**kw):
    """Build a Params from keyword arguments (defaults: a quiet 32^3 NS run)."""
    p = Params()
    defaults = dict(nx=32, ny=32, nz=32, sw_eq=NAVIER_STOKES, dx=1.0, rho=1.0, eta=1.0,
                    kbt=0.0, dt=0.05, a=4.0, a_xi=2.0, lj_epsilon=1.0, lj_powers=0,
                    lj_truncate=1, rotation=0, fixed_particle=0, n_particles=0,
                    n_species=1, g=0.0, g_direction=2, dielectric=0, dielectric_cst=1.0,
                    eps_fluid=80.0, eps_particle_top=2.0, eps_particle_bottom=2.0,
                    potential_iter=1000, potential_tol=1e-10, valency_pos=1.0,
                    valency_neg=-1.0, onsager_pos=1.0, onsager_neg=1.0, debye_length=1.0,
                    elementary_charge=1.0, external_field=0, precision=FP64,
                    solver=SOLVER_REF, per_particle_eps=0)
    mass_ratio = kw.pop("mass_ratio", [1.0] * MAX_SPECIES)
    prop = kw.pop("janus_propulsion", [NO_PROPULSION] * MAX_SPECIES)
    jf = kw.pop("janus_force", [[0.0] * 3] * MAX_SPECIES)
    jt = kw.pop("janus_torque", [[0.0] * 3] * MAX_SPECIES)
    e_ext = kw.pop("e_ext", [0.0, 0.0, 0.0])
    jax = kw.pop("janus_axis", [JANUS_NONE] * MAX_SPECIES)
    qs = kw.pop("surface_charge", [0.0] * MAX_SPECIES)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, v)
    for i in range(MAX_SPECIES):
        p.mass_ratio[i] = mass_ratio[i] if i < len(mass_ratio) else 1.0
        p.janus_propulsion[i] = prop[i] if i < len(prop) else NO_PROPULSION
        p.janus_axis[i] = jax[i] if i < len(jax) else JANUS_NONE
        p.surface_charge[i] = qs[i] if i < len(qs) else 0.0
        for d in range(3):
            p.janus_force[i][d] = jf[i][d] if i < len(jf) else 0.0
            p.janus_torque[i][d] = jt[i][d] if i < len(jt) else 0.0
    for d in range(3):
        p.e_ext[d] = e_ext[d]
    return p


def params_dict(p):
    """Plain-dict copy of a Params (for JSON records)."""
    out = {}
    for name, _ in Params._fields_:
        v = getattr(p, name)
        if isinstance(v, C.Array):
            v = [list(x) if isinstance(x, C.Array) else x for x in v]
        out[name] = v
    return out


def make_particles(x, v=None, spec=None, eps_p=None, q=None):
    """Particle array with positions x (n,3), optional velocities, species,
    per-particle permittivity and orientation quaternions q (n,4) as
    (s, v0, v1, v2); every other field zero, q = identity by default."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    arr = (Particle * max(n, 1))()
    for i in range(n):
        p = arr[i]
        p.spec = 0 if spec is None else int(spec[i])
        for d in range(3):
            p.x[d] = x[i, d]
            p.x_nopbc[d] = x[i, d]
            if v is not None:
                p.v[d] = v[i, d]
        qq = (1.0, 0.0, 0.0, 0.0) if q is None else q[i]
        for a in range(4):
            p.q[a] = float(qq[a])
            p.q_old[a] = float(qq[a])
        p.eps_p = 0.0 if eps_p is None else float(eps_p[i])
    return arr


def particles_to_numpy(arr, n):
    """Dict of (n,3)/(n,4) float64 arrays from a Particle array."""
    out = {}
    for name in PARTICLE_VEC_FIELDS:
        out[name] = np.array([list(getattr(arr[i], name)) for i in range(n)], dtype=np.float64)
    out["spec"] = np.array([arr[i].spec for i in range(n)], dtype=np.int32)
    return out


def field_len(p):
    return p.nx * p.ny * (2 * (p.nz // 2 + 1))
