// particles.cuh -- particle <-> grid transfers, Lennard-Jones forces and the
// FP64 particle integrators.
#pragma once
#include "common.cuh"

namespace icep {

struct PartParams {
  double dx, radius, xi, hxi;
  double L[3];
  int N[3];
  int nzp;
  int rotation;
  int np;
  int np_domain;
  double eps_f;
  double dt;
  double rho;
  double lj_eps, lj_dia, r_cutoff;
  int lj_powers;
  int n_species;
  double imass[ICEP_MAX_SPECIES], imoi[ICEP_MAX_SPECIES];
  double mass_ratio[ICEP_MAX_SPECIES];
  int motor[ICEP_MAX_SPECIES];
  double jforce[ICEP_MAX_SPECIES][3], jtorque[ICEP_MAX_SPECIES][3];
  double g;
  int g_direction;
  int lj_on;
  // Janus permittivity (Make_janus_permittivity_dielectric,
  // operate_dielectric.cxx:208-267): per species the body axis e3 (0, 1, 2
  // for x, y, z; -1 none), eps_ave/eps_delta = (top +- bottom)/2 * Dc and
  // the tanh sharpness 1/DX
  int janus_axis[ICEP_MAX_SPECIES];
  double eps_ave, eps_delta, sharp;
  // surface charge e Q of each species (Make_phi_qq_particle)
  double qe[ICEP_MAX_SPECIES];
  // squared distances outside which no point is in the surface band
  // |r - radius| < hxi (margins far above the rounding of the exact test)
  double band_lo2, band_hi2;
};
// the band bounds of pp from pp.radius and pp.hxi
inline void set_band_bounds(PartParams &pp) {
  const double lo = pp.radius - pp.hxi, hi = pp.radius + pp.hxi;
  pp.band_lo2 = lo > 0.0 ? lo * lo * (1.0 - 1e-12) : 0.0;
  pp.band_hi2 = hi * hi * (1.0 + 1e-12);
}

// The Lennard-Jones constants of Set_global_parameters (input.cxx:404-440)
// into pp: lj_eps, lj_dia = 2 a, lj_powers, the cutoff (2^(1/6), 2^(1/12)
// or 2^(1/18) diameters for LJ_truncate ON; half the smallest box edge, at
// most 2.5 diameters, for OFF; none for NONE) and lj_on. Needs pp.radius,
// pp.dx and pp.N set; shared by contexts and the context-free entry point.
void lj_params_from(const icep_params &p, PartParams &pp);

// Profile scatters over the integration stencil (Particle_domain stencil,
// profile.cxx:25-74), one thread per (particle, stencil point), atomics:
//   PROF_PHI:     out += Phi (Make_phi_particle_sum, make_phi.cxx:229-275)
//   PROF_PHI_SIN: out += Phi_compact_sin; if aux: aux += (eps_p - eps_f) Phi_compact_sin
//                 (Make_phi_sin_primitive, operate_dielectric.cxx:78-120)
//   PROF_JANUS:   out += Phi_compact_sin; aux += Phi_compact_sin (eps_ave +
//                 eps_delta tanh(sharp r.n)), n the particle's Janus axis in
//                 the space frame (Make_janus_permittivity_dielectric,
//                 operate_dielectric.cxx:173-267)
//   PROF_QQ:      out += Phi; aux += e Q DPhi_compact_sin (Make_phi_qq_particle,
//                 operate_electrolyte.cxx:179-218, before its rescaling)
enum { PROF_PHI = 0, PROF_PHI_SIN = 1, PROF_JANUS = 2, PROF_QQ = 3 };
template <typename R>
void scatter_profile(const PartParams &pp, const icep_particle *p, const int *sek, R *out, R *aux, int kind,
                     cudaStream_t s);
// Make_u_particle_sum (make_phi.cxx:329-370)
template <typename R>
void scatter_up(const PartParams &pp, const icep_particle *p, const int *sek, const R *phs, R *u0, R *u1, R *u2,
                cudaStream_t s);
// Make_surface_normal (make_phi.cxx:17-61)
template <typename R>
void scatter_normal(const PartParams &pp, const icep_particle *p, const int *sek, R *s0, R *s1, R *s2,
                    cudaStream_t s);
// Calc_f_hydro_correct_precision (md_force.cxx:340-449); copy_to_1: also
// store into f_hydro1/torque_hydro1 (sp_3d_ns.cxx:69-76)
template <typename R>
void f_hydro(const PartParams &pp, icep_particle *p, const int *sek, const R *phs, const R *u0, const R *u1,
             const R *u2, bool copy_to_1, cudaStream_t s);

// Linked-cell LJ force (md_force.cxx:16-171) added to fr; optional pair list
// (i > j, one entry per visit, so the 2-cells-per-side multiplicity shows).
// work: >= 4*(cells+1) + 2*np ints of device scratch.
int lj_force(const PartParams &pp, icep_particle *p, int *work, int work_ints, int *pairs, int max_pairs,
             int *n_pairs, cudaStream_t s);

// MD_solver_position_Euler/_AB2 (particle_solver.cxx:39-91) with the
// orientation updates (particle_rotation_solver.h:15-39)
void md_position(const PartParams &pp, icep_particle *p, bool ab2, cudaStream_t s);
// MD_solver_velocity_Euler/_AB2_hydro (particle_solver.cxx:109-150,
// 252-295): gravity, self-propulsion, update, reset_Forces. The LJ part of
// Force() must already be in fr.
void md_velocity(const PartParams &pp, icep_particle *p, bool ab2, cudaStream_t s);

}  // namespace icep
