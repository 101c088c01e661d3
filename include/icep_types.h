/*
 * icep_types.h -- plain-C data types shared by the GB300 library's C-ABI
 * (icep_gb300.h) and its callers.
 *
 * Layout conventions follow the reference (KAPSEL-ICEP):
 *   - every grid field is a caller-owned double array [NX][NY][NZ_] with
 *     NZ_ = 2*(NZ/2+1), z fastest, two padding doubles per z row
 *     (alloc_1d_double(NX*NY*NZ_) in the reference, sp_3d_ns.cxx:295-340);
 *   - k-space data are interleaved (re,im) pairs in the same buffer,
 *     half spectrum kz = 0..NZ/2 (fft_wrapper.h:681-723);
 *   - vectors of fields are arrays of separate fields, component-major.
 */
#ifndef ICEP_TYPES_H
#define ICEP_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

#define ICEP_MAX_SPECIES 4

/* Equation type, values of the reference's enum EQ (input.h:46-50). */
enum icep_eq { ICEP_NAVIER_STOKES = 0, ICEP_ELECTROLYTE = 3 };

/* Particle propulsion, values of the reference's enum JP (input.h:56). */
enum icep_propulsion { ICEP_MOTOR = 0, ICEP_NO_PROPULSION = 3 };

/* Arithmetic of the GPU path. FP64 reproduces the reference's FP64 CPU
 * arithmetic; MIXED runs FFTs, advection and inner Krylov sweeps in FP32 and
 * keeps particle integration, the k=0 mode and the Poisson true residual in
 * FP64. */
enum icep_precision { ICEP_FP64 = 0, ICEP_MIXED = 1 };

/* Poisson solver: REF = identity-preconditioned BiCGSTAB with the
 * reference's (Eigen's) stopping and restart rules; SPECTRAL = BiCGSTAB
 * right-preconditioned by the inverse constant-permittivity operator,
 * stopping on the true residual; LEARNED (MIXED precision only) = flexible
 * GMRES whose preconditioner adds a trained U-Net correction to the spectral
 * one, with SPECTRAL as the fallback on stagnation. */
enum icep_solver { ICEP_SOLVER_REF = 0, ICEP_SOLVER_SPECTRAL = 1, ICEP_SOLVER_LEARNED = 2 };

/* Janus axis of a species: the body-frame axis e3 whose rotation by the
 * particle's quaternion separates the eps_particle_top (e3 side) and
 * eps_particle_bottom halves (JAX {x_axis, y_axis, z_axis, no_axis}). */
enum icep_janus_axis { ICEP_JANUS_NONE = 0, ICEP_JANUS_X = 1, ICEP_JANUS_Y = 2, ICEP_JANUS_Z = 3 };

/*
 * Simulation parameters. Field names follow the reference's input.udf keys
 * and globals (input.cxx:286-440 derives the rest):
 *   nx,ny,nz       mesh (NX = 1<<NPX, powers of two, 16..256)
 *   dx,rho,eta,kbt DX, RHO, ETA, kBT
 *   dt             time_increment.manual.delta_t (DT)
 *   a, a_xi        A and A_XI (radius and interface width in units of DX)
 *   lj_*           EPSILON, LJ_powers (0:12:6 1:24:12 2:36:18),
 *                  LJ_truncate (1 ON, 0 OFF, -1 NONE)
 *   species        Component_Number species; per species MASS_RATIOS,
 *                  janus_propulsion, janus_force, janus_torque
 *   dielectric ... constitutive_eq.Electrolyte.* keys
 */
typedef struct icep_params {
  int nx, ny, nz;
  int sw_eq;
  double dx, rho, eta, kbt;
  double dt;
  double a, a_xi;
  double lj_epsilon;
  int lj_powers;
  int lj_truncate;
  int rotation;
  int fixed_particle;
  int n_particles;
  int n_species;
  double mass_ratio[ICEP_MAX_SPECIES];
  int janus_propulsion[ICEP_MAX_SPECIES];
  double janus_force[ICEP_MAX_SPECIES][3];
  double janus_torque[ICEP_MAX_SPECIES][3];
  double g;
  int g_direction;
  /* Electrolyte with Dielectric_property = ON (salt, no surface charge) */
  int dielectric;
  double dielectric_cst;
  double eps_fluid;
  double eps_particle_top;
  double eps_particle_bottom;
  int potential_iter;
  double potential_tol;
  double valency_pos, valency_neg;
  double onsager_pos, onsager_neg;
  double debye_length;
  double elementary_charge;
  int external_field;
  double e_ext[3];
  /* GPU-path options (not reference parameters) */
  int precision;      /* enum icep_precision */
  int solver;         /* enum icep_solver */
  int per_particle_eps; /* 1: use icep_particle.eps_p instead of eps_particle_top */
  /* Janus dielectric particles (Make_janus_permittivity_dielectric,
   * operate_dielectric.cxx:208-267): per species the body axis of the Janus
   * cap, enum icep_janus_axis (the reference's JAX, input.h:55, renumbered so
   * that a zero-initialised struct means no Janus particles). The field is
   * Janus when particle 0's species has an axis (operate_dielectric.cxx:
   * 276-280); then every particle's species needs one. */
  int janus_axis[ICEP_MAX_SPECIES];
  /* switch.FIX_CELL (input.cxx:1603-1625): bit d set keeps the mean flow
   * uk_dc[d] at zero after every fluid update (sp_3d_ns.cxx:30-36) */
  int fix_cell;
  /* Particle_spec[].Surface_charge (input.cxx:1038): all zero (the salt
   * solution path) or all non-zero (Init_rho_ion_dielectric,
   * operate_electrolyte.cxx:912-937): then the charge field adds the
   * particles' surface charge (Conc_k2charge_field, operate_electrolyte.cxx:
   * 45-74) and the ions start with their counterions */
  double surface_charge[ICEP_MAX_SPECIES];
  /* Electric_field.ON.AC (input.cxx:826-845): ac = 1 multiplies E_ext by
   * sin(2 pi frequency t) at the step's time t (Make_Maxwell_force_x_on_fluid,
   * operate_dielectric.cxx:620-627; Add_constant_field_k, fluid_solver.cxx:
   * 231-244; Init_potential_dielectric at t = 0) */
  int ac;
  double frequency;
  /* Add_salt saltfree (input.cxx:751-766): salt_free = 1 runs one ion
   * species, the counterions of the charged particles (N_spec = 1,
   * Valency_counterion, Onsager_coeff_counterion; Init_rho_ion,
   * operate_electrolyte.cxx:738-862); every species needs a surface charge
   * of one sign, opposite to the counterions'. 0: the salt solution. The
   * second concentration field stays zero. */
  int salt_free;
  double valency_counterion;
  double onsager_counterion;
  /* constitutive_eq.Electrolyte.INIT_profile: 0 Uniform, 1 Poisson_Boltzmann
   * (input.cxx:704-715). With charged particles in the salt solution and more
   * than one particle, the uniform ion densities are relaxed towards their
   * steady state before the first step (Set_steadystate_ion_density,
   * operate_electrolyte.cxx:424-457). */
  int poisson_boltzmann;
} icep_params;

/*
 * The per-particle state on the hot path: the subset of the reference's
 * struct Particle (variable.h:27-77) that the spherical-particle step reads
 * or writes. Quaternions are (s, v0, v1, v2).
 */
typedef struct icep_particle {
  int spec;
  int pad_;
  double x[3];
  double x_nopbc[3];
  double v[3];
  double v_old[3];
  double omega[3];
  double omega_old[3];
  double f_hydro[3];
  double f_hydro_previous[3];
  double f_hydro1[3];
  double fr[3];
  double fr_previous[3];
  double torque_hydro[3];
  double torque_hydro_previous[3];
  double torque_hydro1[3];
  double torque_r[3];
  double torque_r_previous[3];
  double q[4];
  double q_old[4];
  double eps_p; /* per-particle permittivity (extension; reference: global) */
} icep_particle;

#ifdef __cplusplus
}
#endif
#endif
