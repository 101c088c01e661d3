/*
 * ref_harness.cxx -- drives the reference's own hot-path object code.
 *
 * TEST INFRASTRUCTURE ONLY. Linked with the reference sources (compiled in
 * place by oracle/ref/Makefile) into oracle/_ref/libkapsel_ref.so. Used to
 * generate golden fixtures and to validate the C restatement; never part of
 * the product.
 *
 * What this file supplies:
 *   - definitions of the globals that the reference defines in input.cxx
 *     (input.cxx:18-280), filled the way Set_global_parameters does
 *     (input.cxx:286-440) instead of by parsing a UDF file;
 *   - the allocation and initialisation sequence of main()
 *     (sp_3d_ns.cxx:295-340 Mem_alloc_var, :404-457 init) and the
 *     particle reset of Init_Particle (init_particle.cxx:380-425);
 *   - the call order of Time_evolution_hydro (sp_3d_ns.cxx:24-186) for the
 *     Navier_Stokes and Electrolyte+Dielectric (no surface charge) cases;
 *   - kref_* C entry points for ctypes.
 */
#include "fluid_solver.h"
#include "operate_dielectric.h"
#include "operate_electrolyte.h"
#include "md_force.h"
#include "particle_solver.h"
#include "make_phi.h"
#include "f_particle.h"
#include "init_fluid.h"
#include "profile.h"
#include "fft_wrapper.h"
#include "operate_omega.h"
#include "solute_rhs.h"
#include "avs_output.h"
#include "avs_output_p.h"

#include "../../include/icep_types.h"

/* ---- globals defined in the reference's input.cxx (types from input.h) -- */
EQ SW_EQ;
PT SW_PT;
int Ns[DIM];
int Ns_shear[DIM];
int HNs[DIM];
int TRNs[DIM];
int N2s[DIM];
int HN2s[DIM];
int &NX = Ns[0];
int &NY = Ns[1];
int &NZ = Ns[2];
int &HNX = HNs[0];
int &HNY = HNs[1];
int &TRN_X = TRNs[0];
int &TRN_Y = TRNs[1];
int &TRN_Z = TRNs[2];
int HNZ_;
int NZ_;
double L[DIM];
double L_particle[DIM];
double &LX = L[0];
double &LY = L[1];
double &LZ = L[2];
double dev_shear_stress[2];
double rigid_dev_shear_stress[2];
double &dev_shear_stress_lj = dev_shear_stress[0];
double &dev_shear_stress_rot = dev_shear_stress[1];
double &rigid_dev_shear_stress_lj = rigid_dev_shear_stress[0];
double &rigid_dev_shear_stress_rot = rigid_dev_shear_stress[1];
JAX *janus_axis;
JP *janus_propulsion;
double **janus_force;
double **janus_torque;
double A, A_R_cutoff, A_XI, Angular_Frequency;
int *Beads_Numbers, *Chain_Numbers;
int Component_Number;
double DX, DX3, Debye_length, Dielectric_cst;
int Dielectric;
double EPSILON, ETA;
double E_ext[DIM];
double Elementary_charge = 1.;
int External_field, Fixed_particle;
int FIX_CELL, FIX_CELLxyz[DIM];
double G;
int G_direction;
double HXI;
double *IMASS, *IMOI, *MASS_RATIOS, *RHO_particle;
double Ivolume, LJ_dia;
int LJ_powers, LJ_truncate;
int MaxIter_potential;
double NU;
int N_spec;
double Onsager_coeff_counterion, Onsager_coeff_negative_ion, Onsager_coeff_positive_ion;
int Particle_Number;
int *Particle_Numbers;
int *Particle_RigidID;
int Poisson_Boltzmann;
double RADIUS, RHO;
int ROTATION;
int *RigidID_Components;
double *Rigid_IMasses, *Rigid_Masses;
double ***Rigid_IMoments, ***Rigid_Moments, ***Rigid_Moments_body;
int **Rigid_Motions_omega, **Rigid_Motions_vel;
int Rigid_Number;
int *Rigid_Particle_Cumul;
double SIGMA;
int SW_JANUS_MOTOR;
int Shear_AC;
double Shear_frequency, Shear_rate, Shear_rate_eff;
double *Surface_charge, *Surface_charge_e;
double Tol_potential;
double Valency_counterion, Valency_negative_ion, Valency_positive_ion;
double WAVE_X, WAVE_Y, WAVE_Z;
double XI;
double degree_oblique;
double eps_fluid, eps_particle_bottom, eps_particle_top;
double kBT;
int AC;
/* the AVS writers' globals (input.cxx) */
char Out_dir[256], Out_name[256];
OUTFORMAT SW_OUTFORMAT = OUT_NONE;
int Num_snap;
double **GRvecs, **GRvecs_body;
double **forceGrs, **forceGrs_previous, **forceGs, **forceGs_previous;
double **omegaGs, **omegaGs_old, **torqueGrs, **torqueGrs_previous;
double **torqueGs, **torqueGs_previous, **velocityGs, **velocityGs_old;
double **xGs, **xGs_nopbc, **xGs_previous;

/* defined in operate_dielectric.cxx:18-22 without a header declaration */
extern void (*Charge_field2potential_dielectric)(double *, double *, double *, double *, double[]);

/* ---- harness state (main()'s locals, sp_3d_ns.cxx:404-420) ---------------- */
static double *zeta[DIM - 1];
static double *c1_absent = nullptr;  // c1 of a salt-free run (N_spec = 1)
static double uk_dc[DIM];
static CTime jikan;
static Particle *particles = nullptr;
static double *rho_free_buf = nullptr; /* free charge density for isolated calls */
static double *work_buf = nullptr;
static bool ready = false;
static bool spectral_solve = false; /* icep_params.solver == ICEP_SOLVER_SPECTRAL */

/*
 * The plain method of the GPU path, installed in the reference's own solver
 * seam (the Charge_field2potential_dielectric function pointer,
 * operate_dielectric.cxx:18-22, which the reference provides so that the
 * solve can be swapped) when a fixture asks for a tolerance that the
 * reference's identity-preconditioned BiCGSTAB cannot reach on an
 * inconsistent periodic system: BiCGSTAB right-preconditioned by the
 * constant-permittivity spectral inverse y(k) = -x(k) IK2(k) / eps_ref
 * (eps_ref = mean eps, IK2 the reference's 1/K^2 table, fft_wrapper.cxx:
 * 47-87), b projected to mean zero, convergence confirmed on the true
 * residual |b - A x| <= tol |b|, the retry from a zero guess of
 * Charge_field2potential_dielectric_LO (operate_dielectric.cxx:563-570).
 * Everything else is the reference's: Build_rhs, Ax, the Ooura transforms.
 */
static void spectral_precond(const std::vector<double> &x, std::vector<double> &y, double eref) {
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY; j++) {
      for (int k = 0; k < NZ; k++) work_v1[(i * NY * NZ_) + (j * NZ_) + k] = x[(i * NY + j) * NZ + k];
      for (int k = NZ; k < NZ_; k++) work_v1[(i * NY * NZ_) + (j * NZ_) + k] = 0.0;
    }
  A2a_k(work_v1);
  for (int im = 0; im < NX * NY * NZ_; im++) work_v1[im] *= -IK2[im] / eref;
  A_k2a(work_v1);
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ; k++) y[(i * NY + j) * NZ + k] = work_v1[(i * NY * NZ_) + (j * NZ_) + k];
}

static double vdot(const std::vector<double> &a, const std::vector<double> &b) {
  double s = 0.0;
  for (size_t k = 0; k < a.size(); k++) s += a[k] * b[k];
  return s;
}

static long spectral_bicgstab(std::vector<double> b, std::vector<double> &x, double eref, double *err) {
  const size_t n = b.size();
  double mean = 0.0;
  for (size_t k = 0; k < n; k++) mean += b[k];
  mean /= (double)n;
  for (size_t k = 0; k < n; k++) b[k] -= mean;
  std::vector<double> r(n), r0(n), v(n, 0.0), p(n, 0.0), s(n), t(n), y(n), z(n);
  auto matvec = [&](const std::vector<double> &in, std::vector<double> &out) {
    ++Eigen::shim_stats::matvecs();
    Ax(in.data(), out.data());
  };
  matvec(x, t);
  for (size_t k = 0; k < n; k++) r[k] = b[k] - t[k];
  r0 = r;
  double r0_sq = vdot(r0, r0), b_sq = vdot(b, b);
  long i = 0;
  if (b_sq == 0.0) {
    std::fill(x.begin(), x.end(), 0.0);
    *err = 0.0;
    return 0;
  }
  double rho = 1, alpha = 1, w = 1, rr = r0_sq, rho_new = r0_sq;
  const double tol2 = Tol_potential * Tol_potential * b_sq;
  const double eps2 = std::numeric_limits<double>::epsilon() * std::numeric_limits<double>::epsilon();
  long restarts = 0;
  while (i < MaxIter_potential) {
    if (!(rr > tol2)) {
      matvec(x, t);
      for (size_t k = 0; k < n; k++) r[k] = b[k] - t[k];
      rr = vdot(r, r);
      if (!(rr > tol2)) break;
      r0 = r;
      r0_sq = rho_new = rr;
      std::fill(v.begin(), v.end(), 0.0);
      std::fill(p.begin(), p.end(), 0.0);
      rho = alpha = w = 1;
    }
    const double rho_old = rho;
    rho = rho_new;
    if (std::fabs(rho) < eps2 * r0_sq) {
      matvec(x, t);
      for (size_t k = 0; k < n; k++) r[k] = b[k] - t[k];
      r0 = r;
      rho = r0_sq = vdot(r, r);
      if (restarts++ == 0) i = 0;
    }
    const double beta = (rho / rho_old) * (alpha / w);
    for (size_t k = 0; k < n; k++) p[k] = r[k] + beta * (p[k] - w * v[k]);
    spectral_precond(p, y, eref);
    matvec(y, v);
    alpha = rho / vdot(r0, v);
    for (size_t k = 0; k < n; k++) s[k] = r[k] - alpha * v[k];
    spectral_precond(s, z, eref);
    matvec(z, t);
    const double tt = vdot(t, t);
    w = (tt > 0.0) ? vdot(t, s) / tt : 0.0;
    for (size_t k = 0; k < n; k++) x[k] += alpha * y[k] + w * z[k];
    for (size_t k = 0; k < n; k++) r[k] = s[k] - w * t[k];
    rho_new = vdot(r0, r);
    rr = vdot(r, r);
    ++i;
  }
  *err = std::sqrt(rr / b_sq);
  return i;
}

static void potential_spectral(double *free_charge_density, double *potential, double *eps, double *rhs,
                               double external_e_field[]) {
  Reset_phi(rhs);
  Build_rhs(rhs, free_charge_density, eps, external_e_field);
  const size_t n = (size_t)NX * NY * NZ;
  std::vector<double> b(n), x(n);
  double eref = 0.0;
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ; k++) {
        const int im = (i * NY * NZ_) + (j * NZ_) + k;
        b[(i * NY + j) * NZ + k] = rhs[im];
        x[(i * NY + j) * NZ + k] = potential[im];
        eref += eps[im];
      }
  eref /= (double)n;
  double err = 0.0;
  long it = spectral_bicgstab(b, x, eref, &err);
  if (it == MaxIter_potential) {
    std::fill(x.begin(), x.end(), 0.0);
    it = spectral_bicgstab(b, x, eref, &err);
  }
  Eigen::shim_stats::iterations() = it;
  Eigen::shim_stats::error() = err;
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ; k++) potential[(i * NY * NZ_) + (j * NZ_) + k] = x[(i * NY + j) * NZ + k];
}

static double *dalloc(int n) {
  double *p = alloc_1d_double(n);
  for (int i = 0; i < n; i++) p[i] = 0.0;
  return p;
}

/* Set_global_parameters (input.cxx:286-440) restricted to what the path reads. */
static void set_globals(const icep_params *q) {
  Ns[0] = q->nx; Ns[1] = q->ny; Ns[2] = q->nz;
  for (int d = 0; d < DIM; d++) Ns_shear[d] = Ns[d];
  SW_EQ = (q->sw_eq == ICEP_ELECTROLYTE) ? Electrolyte : Navier_Stokes;
  SW_PT = spherical_particle;
  DX = q->dx; RHO = q->rho; ETA = q->eta; kBT = q->kbt;
  A = q->a; A_XI = q->a_xi;
  XI = A_XI * DX; RADIUS = A * DX; SIGMA = 2.0 * RADIUS;
  EPSILON = q->lj_epsilon; LJ_powers = q->lj_powers; LJ_truncate = q->lj_truncate;
  ROTATION = q->rotation; Fixed_particle = q->fixed_particle;
  G = q->g; G_direction = q->g_direction;
  Component_Number = q->n_species;
  Particle_Numbers = (int *)calloc(Component_Number, sizeof(int));
  MASS_RATIOS = (double *)calloc(Component_Number, sizeof(double));
  IMASS = (double *)calloc(Component_Number, sizeof(double));
  IMOI = (double *)calloc(Component_Number, sizeof(double));
  RHO_particle = (double *)calloc(Component_Number, sizeof(double));
  Surface_charge = (double *)calloc(Component_Number, sizeof(double));
  Surface_charge_e = (double *)calloc(Component_Number, sizeof(double));
  janus_axis = (JAX *)calloc(Component_Number, sizeof(JAX));
  janus_propulsion = (JP *)calloc(Component_Number, sizeof(JP));
  janus_force = (double **)calloc(Component_Number, sizeof(double *));
  janus_torque = (double **)calloc(Component_Number, sizeof(double *));
  SW_JANUS_MOTOR = 0;
  FIX_CELL = 0;
  for (int d = 0; d < DIM; d++) {  // switch.FIX_CELL (input.cxx:1603-1625)
    FIX_CELLxyz[d] = (q->fix_cell >> d) & 1;
    FIX_CELL |= FIX_CELLxyz[d];
  }
  for (int i = 0; i < Component_Number; i++) {
    MASS_RATIOS[i] = q->mass_ratio[i];
    Surface_charge[i] = q->surface_charge[i];
    RHO_particle[i] = MASS_RATIOS[i] * RHO;
    double mass = RHO_particle[i] * 4. / 3. * M_PI * POW3(RADIUS);
    IMASS[i] = 1. / mass;
    IMOI[i] = 1. / (2. / 5. * mass * SQ(RADIUS));
    // icep_janus_axis (0 none, 1..3 x..z) -> the reference's JAX (input.h:55)
    switch (q->janus_axis[i]) {
      case ICEP_JANUS_X: janus_axis[i] = x_axis; break;
      case ICEP_JANUS_Y: janus_axis[i] = y_axis; break;
      case ICEP_JANUS_Z: janus_axis[i] = z_axis; break;
      default: janus_axis[i] = no_axis;
    }
    janus_propulsion[i] = (q->janus_propulsion[i] == ICEP_MOTOR) ? motor : no_propulsion;
    if (janus_propulsion[i] == motor) SW_JANUS_MOTOR = 1;
    janus_force[i] = (double *)calloc(DIM, sizeof(double));
    janus_torque[i] = (double *)calloc(DIM, sizeof(double));
    for (int d = 0; d < DIM; d++) {
      janus_force[i][d] = q->janus_force[i][d];
      janus_torque[i][d] = q->janus_torque[i][d];
    }
  }
  Particle_Number = q->n_particles;
  NU = ETA / RHO;
  DX3 = DX * DX * DX;
  HNZ_ = NZ / 2 + 1;
  NZ_ = 2 * HNZ_;
  for (int d = 0; d < DIM; d++) {
    HNs[d] = Ns[d] / 2;
    TRNs[d] = (Ns[d] + 2) / 3;
    N2s[d] = Ns[d] * 2;
    HN2s[d] = Ns[d];
    L[d] = Ns[d] * DX;
    L_particle[d] = L[d];
  }
  WAVE_X = PI2 / LX; WAVE_Y = PI2 / LY; WAVE_Z = PI2 / LZ;
  /* LJ cutoff (input.cxx:1530-1546) and LJ_dia (input.cxx:404-424) */
  if (LJ_truncate > 0) {
    A_R_cutoff = (LJ_powers == 0) ? pow(2., 1. / 6.) : (LJ_powers == 1) ? pow(2., 1. / 12.) : pow(2., 1. / 18.);
  } else if (LJ_truncate == 0) {
    int nmin = MIN(NX, MIN(NY, NZ));
    A_R_cutoff = MIN(nmin * DX * .5 / SIGMA, 2.5);
  } else {
    A_R_cutoff = 0.;
  }
  LJ_dia = SIGMA;
  HXI = XI * 0.5;
  Ivolume = 1. / (LX * LY * LZ);
  /* electrolyte */
  Dielectric = q->dielectric;
  Dielectric_cst = q->dielectric_cst;
  eps_fluid = q->eps_fluid;
  eps_particle_top = q->eps_particle_top;
  eps_particle_bottom = q->eps_particle_bottom;
  MaxIter_potential = q->potential_iter;
  Tol_potential = q->potential_tol;
  Valency_positive_ion = q->valency_pos;
  Valency_negative_ion = q->valency_neg;
  Onsager_coeff_positive_ion = q->onsager_pos;
  Onsager_coeff_negative_ion = q->onsager_neg;
  Debye_length = q->debye_length;
  Elementary_charge = q->elementary_charge;
  External_field = q->external_field;
  for (int d = 0; d < DIM; d++) E_ext[d] = q->e_ext[d];
  AC = q->ac ? 1 : 0;  // Electric_field.ON.AC (input.cxx:826-845, 370-374)
  Angular_Frequency = 2.0 * M_PI * q->frequency;
  N_spec = q->salt_free ? 1 : 2;  // Add_salt saltfree / salt (input.cxx:751-770)
  Valency_counterion = q->valency_counterion;
  Onsager_coeff_counterion = q->onsager_counterion;
  Poisson_Boltzmann = q->poisson_boltzmann;  // INIT_profile (input.cxx:704-715)
  Rigid_Number = 0;
  degree_oblique = 0.0;
}

/* Mem_alloc_var (sp_3d_ns.cxx:295-340) */
static void mem_alloc() {
  Mem_alloc_NS_solver();
  if (SW_EQ == Electrolyte) {
    Mem_alloc_charge();
    if (Dielectric) Mem_alloc_potential();
  }
  Mem_alloc_f_particle();
  for (int d = 0; d < DIM - 1; d++) zeta[d] = dalloc(NX * NY * NZ_);
  u = (double **)malloc(sizeof(double *) * DIM);
  up = (double **)malloc(sizeof(double *) * DIM);
  work_v3 = (double **)malloc(sizeof(double *) * DIM);
  for (int d = 0; d < DIM; d++) {
    u[d] = dalloc(NX * NY * NZ_);
    up[d] = dalloc(NX * NY * NZ_);
    work_v3[d] = dalloc(NX * NY * NZ_);
  }
  work_v2 = (double **)malloc(sizeof(double *) * (DIM - 1));
  for (int d = 0; d < DIM - 1; d++) work_v2[d] = dalloc(NX * NY * NZ_);
  phi = dalloc(NX * NY * NZ_);
  phi_sum = dalloc(NX * NY * NZ_);
  rhop = dalloc(NX * NY * NZ_);
  work_v1 = dalloc(NX * NY * NZ_);
  Hydro_force = dalloc(NX * NY * NZ_);
  Hydro_force_new = dalloc(NX * NY * NZ_);
  rho_free_buf = dalloc(NX * NY * NZ_);
  work_buf = dalloc(NX * NY * NZ_);
  /* The reference's alloc_1d_double does not clear memory; large arrays come
   * from fresh (zero) pages. Clear the ones the path reads before writing so
   * that every run starts from the same state. */
  const size_t bytes = sizeof(double) * NX * NY * NZ_;
  for (int d = 0; d < DIM - 1; d++) { memset(f_ns0[d], 0, bytes); memset(f_ns1[d], 0, bytes); }
  for (int d = 0; d < DIM; d++) memset(f_particle[d], 0, bytes);
  if (SW_EQ == Electrolyte) {
    for (int n = 0; n < N_spec; n++) {
      memset(Concentration[n], 0, bytes);
      memset(Concentration_rhs0[n], 0, bytes);
      memset(Concentration_rhs1[n], 0, bytes);
    }
    for (int d = 0; d < DIM; d++) memset(Surface_normal[d], 0, bytes);
    if (N_spec == 1) {  // the registry's c1 of a salt-free run: zeros
      c1_absent = dalloc(NX * NY * NZ_);
      memset(c1_absent, 0, bytes);
    }
    if (Dielectric) {
      memset(Potential, 0, bytes);
      memset(epsilon, 0, bytes);
      for (int d = 0; d < DIM; d++) memset(grad_epsilon[d], 0, bytes);
    }
  }
}

static void to_particle(const icep_particle *s, Particle *p) {
  p->spec = s->spec;
  for (int d = 0; d < DIM; d++) {
    p->x[d] = s->x[d]; p->x_nopbc[d] = s->x_nopbc[d];
    p->v[d] = s->v[d]; p->v_old[d] = s->v_old[d];
    p->omega[d] = s->omega[d]; p->omega_old[d] = s->omega_old[d];
    p->f_hydro[d] = s->f_hydro[d]; p->f_hydro_previous[d] = s->f_hydro_previous[d];
    p->f_hydro1[d] = s->f_hydro1[d];
    p->fr[d] = s->fr[d]; p->fr_previous[d] = s->fr_previous[d];
    p->torque_hydro[d] = s->torque_hydro[d]; p->torque_hydro_previous[d] = s->torque_hydro_previous[d];
    p->torque_hydro1[d] = s->torque_hydro1[d];
    p->torque_r[d] = s->torque_r[d]; p->torque_r_previous[d] = s->torque_r_previous[d];
    p->f_slip[d] = 0.0; p->f_slip_previous[d] = 0.0;
    p->torque_slip[d] = 0.0; p->torque_slip_previous[d] = 0.0;
  }
  qtn_init(p->q, s->q[0], s->q[1], s->q[2], s->q[3]);
  qtn_init(p->q_old, s->q_old[0], s->q_old[1], s->q_old[2], s->q_old[3]);
}

static void from_particle(const Particle *p, icep_particle *s) {
  s->spec = p->spec;
  for (int d = 0; d < DIM; d++) {
    s->x[d] = p->x[d]; s->x_nopbc[d] = p->x_nopbc[d];
    s->v[d] = p->v[d]; s->v_old[d] = p->v_old[d];
    s->omega[d] = p->omega[d]; s->omega_old[d] = p->omega_old[d];
    s->f_hydro[d] = p->f_hydro[d]; s->f_hydro_previous[d] = p->f_hydro_previous[d];
    s->f_hydro1[d] = p->f_hydro1[d];
    s->fr[d] = p->fr[d]; s->fr_previous[d] = p->fr_previous[d];
    s->torque_hydro[d] = p->torque_hydro[d]; s->torque_hydro_previous[d] = p->torque_hydro_previous[d];
    s->torque_hydro1[d] = p->torque_hydro1[d];
    s->torque_r[d] = p->torque_r[d]; s->torque_r_previous[d] = p->torque_r_previous[d];
  }
  s->q[0] = p->q.s; s->q[1] = p->q.v[0]; s->q[2] = p->q.v[1]; s->q[3] = p->q.v[2];
  s->q_old[0] = p->q_old.s; s->q_old[1] = p->q_old.v[0];
  s->q_old[2] = p->q_old.v[1]; s->q_old[3] = p->q_old.v[2];
}

/* Time_evolution_hydro (sp_3d_ns.cxx:24-186) for spherical particles without
 * slip, thermostat, pinning or shear. */
static void time_evolution_hydro() {
  const Index_range *ijk_range = ijk_range_two_third_filter;
  const int n_ijk_range = n_ijk_range_two_third_filter;
  if (SW_EQ == Navier_Stokes) {
    NS_solver_slavedEuler(zeta, jikan, uk_dc, ijk_range, n_ijk_range, particles);
  } else {
    NSsolute_solver_Euler(zeta, jikan, uk_dc, Concentration, particles, ijk_range, n_ijk_range);
  }
  if (FIX_CELL) {  // sp_3d_ns.cxx:30-36
    for (int d = 0; d < DIM; d++)
      if (FIX_CELLxyz[d]) uk_dc[d] = 0.0;
  }
  for (int d = 0; d < (DIM - 1); d++) Truncate_two_third_rule(zeta[d]);
  Zeta_k2u(zeta, uk_dc, u);
  if (!Fixed_particle) {
    if (jikan.ts == 0) MD_solver_position_Euler(particles, jikan);
    else MD_solver_position_AB2(particles, jikan);
  }
  Reset_phi(phi);
  Reset_phi(phi_sum);
  Make_phi_particle_sum(phi, phi_sum, particles);
  if (SW_EQ == Electrolyte) {
    Reset_u(up);
    Reset_u(f_particle);
    Calc_f_hydro_correct_precision(particles, phi_sum, u, jikan);
    for (int n = 0; n < Particle_Number; n++)
      for (int d = 0; d < DIM; d++) {
        particles[n].f_hydro1[d] = particles[n].f_hydro[d];
        particles[n].torque_hydro1[d] = particles[n].torque_hydro[d];
      }
    Make_Maxwell_force_x_on_fluid(f_particle, particles, Concentration, up[0], Potential, epsilon,
                                  grad_epsilon, jikan);
    double dmy = jikan.dt_fluid / RHO;
    for (int i = 0; i < NX; i++)
      for (int j = 0; j < NY; j++)
        for (int k = 0; k < NZ; k++) {
          int im = (i * NY * NZ_) + (j * NZ_) + k;
          u[0][im] += (f_particle[0][im] * dmy);
          u[1][im] += (f_particle[1][im] * dmy);
          u[2][im] += (f_particle[2][im] * dmy);
        }
    Solenoidal_u(u);
  }
  Reset_u(up);
  Calc_f_hydro_correct_precision(particles, phi_sum, u, jikan);
  if (!Fixed_particle) {
    if (jikan.ts == 0) MD_solver_velocity_Euler(particles, jikan);
    else MD_solver_velocity_AB2_hydro(particles, jikan);
  }
  Reset_u(up);
  Make_u_particle_sum(up, phi_sum, particles);
  Make_f_particle_dt_sole(f_particle, u, up, phi);
  Add_f_particle(u, f_particle);
  U2zeta_k(zeta, uk_dc, u);
}

extern "C" {

/* Statistics of the last BiCGSTAB solve, recorded by the shim. */
long kref_last_iterations() { return Eigen::shim_stats::iterations(); }
double kref_last_error() { return Eigen::shim_stats::error(); }
long kref_matvec_count() { return Eigen::shim_stats::matvecs(); }

int kref_setup(const icep_params *q, const icep_particle *p, int np) {
  set_globals(q);
  if (np != Particle_Number) return 1;
  Init_fft();
  mem_alloc();
  jikan.ts = 0; jikan.time = 0.0;
  jikan.dt_fluid = q->dt; jikan.hdt_fluid = q->dt * 0.5;
  jikan.dt_md = q->dt; jikan.hdt_md = q->dt * 0.5;
  particles = new Particle[Particle_Number > 0 ? Particle_Number : 1];
  Particle_domain(Phi, NP_domain, Sekibun_cell);
  Angular2v = ROTATION ? Angular2v_rot_on : Angular2v_rot_off;
  /* selected in Init_potential_dielectric (operate_dielectric.cxx:592);
   * set here too so that isolated calls can use it; a SPECTRAL case swaps in
   * potential_spectral through the same pointer */
  spectral_solve = (q->solver == ICEP_SOLVER_SPECTRAL);
  Charge_field2potential_dielectric =
      spectral_solve ? potential_spectral : Charge_field2potential_dielectric_LO;
  for (int n = 0; n < Particle_Number; n++) to_particle(&p[n], &particles[n]);
  for (int n = 0; n < Particle_Number; n++)  // Particle_Numbers per species (input.cxx:1036)
    if (particles[n].spec >= 0 && particles[n].spec < Component_Number) Particle_Numbers[particles[n].spec]++;
  ready = true;
  return 0;
}

int kref_np_domain() { return NP_domain; }
void kref_sekibun(int *cells) {
  for (int m = 0; m < NP_domain; m++)
    for (int d = 0; d < DIM; d++) cells[3 * m + d] = Sekibun_cell[m][d];
}

/* main()'s initialisation after Init_Particle (sp_3d_ns.cxx:425-457). */
void kref_init_state() {
  for (int n = 0; n < Particle_Number; n++)
    for (int d = 0; d < DIM; d++) particles[n].x_nopbc[d] = particles[n].x[d];
  Init_zeta_k(zeta, uk_dc);
  Reset_phi_u(phi, up);
  Reset_phi(phi_sum);
  Make_phi_particle_sum(phi, phi_sum, particles);
  Make_u_particle_sum(up, phi_sum, particles);
  Zeta_k2u(zeta, uk_dc, u);
  Make_f_particle_dt_sole(f_particle, u, up, phi);
  Add_f_particle(u, f_particle);
  U2zeta_k(zeta, uk_dc, u);
  for (int d = 0; d < DIM; d++) uk_dc[d] = .0;
  if (SW_EQ == Electrolyte && Dielectric) {
    Reset_u(grad_epsilon);
    Init_rho_ion_dielectric(Concentration, particles, jikan);
    if (!spectral_solve) {
      Init_potential_dielectric(particles, grad_epsilon[2], grad_epsilon[0], Concentration, grad_epsilon[1],
                                Potential, epsilon, jikan);
    } else {
      /* Init_potential_dielectric (operate_dielectric.cxx:574-609) with the
       * solver pointer left at potential_spectral (the reference's version
       * assigns Charge_field2potential_dielectric_LO before its solve) */
      double external[DIM];
      for (int d = 0; d < DIM; d++) external[d] = E_ext[d] * (AC ? sin(Angular_Frequency * jikan.time) : 1.0);
      Make_dielectric_field(particles, epsilon, grad_epsilon[2], eps_particle_top, eps_particle_bottom, eps_fluid);
      if (have_surface_charge)
        Conc_k2charge_field(particles, Concentration, grad_epsilon[1], grad_epsilon[2], grad_epsilon[0]);
      else
        Conc_k2charge_field_no_surfase_charge(particles, Concentration, grad_epsilon[1], grad_epsilon[2],
                                              grad_epsilon[0]);
      potential_spectral(grad_epsilon[1], Potential, epsilon, grad_epsilon[2], external);
    }
  }
}

/* n steps of the main loop body (sp_3d_ns.cxx:524-525). */
void kref_step(int n) {
  for (int s = 0; s < n; s++) {
    time_evolution_hydro();
    jikan.time += jikan.dt_fluid;
    jikan.ts++;
  }
}

void kref_set_ts(int ts, double time) { jikan.ts = ts; jikan.time = time; }

void kref_get_particles(icep_particle *p) {
  for (int n = 0; n < Particle_Number; n++) from_particle(&particles[n], &p[n]);
}
void kref_set_particles(const icep_particle *p) {
  for (int n = 0; n < Particle_Number; n++) to_particle(&p[n], &particles[n]);
}

/* Field registry. */
enum {
  F_ZETA0 = 0, F_ZETA1, F_U0, F_U1, F_U2, F_UP0, F_UP1, F_UP2, F_PHI, F_PHI_SUM,
  F_F0, F_F1, F_F2, F_POT, F_EPS, F_GE0, F_GE1, F_GE2, F_C0, F_C1, F_RHO, F_WORK,
  F_SN0, F_SN1, F_SN2, F_NS0_0, F_NS0_1, F_NS1_0, F_NS1_1, F_COUNT
};
static double *field_ptr(int id) {
  switch (id) {
    case F_ZETA0: return zeta[0];
    case F_ZETA1: return zeta[1];
    case F_U0: case F_U1: case F_U2: return u[id - F_U0];
    case F_UP0: case F_UP1: case F_UP2: return up[id - F_UP0];
    case F_PHI: return phi;
    case F_PHI_SUM: return phi_sum;
    case F_F0: case F_F1: case F_F2: return f_particle[id - F_F0];
    case F_POT: return Potential;
    case F_EPS: return epsilon;
    case F_GE0: case F_GE1: case F_GE2: return grad_epsilon ? grad_epsilon[id - F_GE0] : nullptr;
    case F_C0: return Concentration ? Concentration[0] : nullptr;
    case F_C1: return Concentration ? (N_spec > 1 ? Concentration[1] : c1_absent) : nullptr;
    case F_RHO: return rho_free_buf;
    case F_WORK: return work_buf;
    case F_SN0: case F_SN1: case F_SN2: return Surface_normal ? Surface_normal[id - F_SN0] : nullptr;
    case F_NS0_0: return f_ns0[0];
    case F_NS0_1: return f_ns0[1];
    case F_NS1_0: return f_ns1[0];
    case F_NS1_1: return f_ns1[1];
  }
  return nullptr;
}
int kref_get_field(int id, double *out) {
  double *f = field_ptr(id);
  if (!f) return 1;
  memcpy(out, f, sizeof(double) * NX * NY * NZ_);
  return 0;
}
int kref_set_field(int id, const double *in) {
  double *f = field_ptr(id);
  if (!f) return 1;
  memcpy(f, in, sizeof(double) * NX * NY * NZ_);
  return 0;
}
void kref_get_uk_dc(double *o) { for (int d = 0; d < DIM; d++) o[d] = uk_dc[d]; }
void kref_set_uk_dc(const double *o) { for (int d = 0; d < DIM; d++) uk_dc[d] = o[d]; }

/* In-place FFTs on a caller buffer of NX*NY*NZ_ doubles. */
void kref_a2a_k(double *a) { A2a_k(a); }
void kref_a_k2a(double *a) { A_k2a(a); }

/* Isolated reference calls on the registry fields. */
enum {
  C_ZETA_K2U_K = 1, C_U_K2ZETA_K, C_U2ADVECTION_K, C_SOLENOIDAL_U, C_NS_SLAVED_EULER,
  C_MAKE_PHI_SUM, C_MAKE_U_SUM, C_F_HYDRO, C_LJ, C_POS_EULER, C_POS_AB2, C_VEL_EULER,
  C_VEL_AB2, C_DIELECTRIC_FIELD, C_BUILD_RHS, C_SOLVE_POTENTIAL, C_MAXWELL, C_NSSOLUTE_EULER,
  C_SURFACE_NORMAL, C_F_PARTICLE_SOLE, C_TRUNCATE, C_CHARGE_FIELD, C_INIT_ION, C_ZETA_K2U,
  C_CHARGE_OUTPUT
};

/* The fields Output_dielectric_charge_field_data computes (output.cxx:
 * 262-320) with vel, phi and charge printed, restated around the reference's
 * own Zeta_k2u, Make_phi_qq_particle and FFTs (output.cxx itself needs the
 * writers): u -> u0..u2, phi, up0 surface charge, up1 solute charge, up2 eps.
 * The concentrations go to real space and back, as there. */
static void charge_output() {
  Zeta_k2u(zeta, uk_dc, u);
  Reset_phi(phi);
  Reset_phi(up[0]);
  Make_phi_qq_particle(phi, up[0], particles);
  for (int n = 0; n < N_spec; n++) A_k2a(Concentration[n]);
  const double area = PI4 * SQ(RADIUS);
  for (int i = 0; i < NX; i++)
    for (int j = 0; j < NY; j++)
      for (int k = 0; k < NZ; k++) {
        const int im = (i * NY * NZ_) + (j * NZ_) + k;
        double q = 0.0;
        for (int n = 0; n < N_spec; n++) q += Elementary_charge * Valency[n] * Concentration[n][im];
        up[0][im] *= area;
        up[1][im] = q * (1.0 - phi[im]);
        up[2][im] = epsilon[im];
      }
  for (int n = 0; n < N_spec; n++) A2a_k(Concentration[n]);
}
int kref_call(int fn) {
  const Index_range *ijk_range = ijk_range_two_third_filter;
  const int n_ijk_range = n_ijk_range_two_third_filter;
  switch (fn) {
    case C_ZETA_K2U_K: Zeta_k2u_k(zeta, uk_dc, u); break;
    case C_ZETA_K2U: Zeta_k2u(zeta, uk_dc, u); break;
    case C_U_K2ZETA_K: U_k2zeta_k(u, zeta, uk_dc); break;
    case C_U2ADVECTION_K: U2advection_k(u, f_ns0); break;
    case C_SOLENOIDAL_U: Solenoidal_u(u); break;
    case C_NS_SLAVED_EULER: NS_solver_slavedEuler(zeta, jikan, uk_dc, ijk_range, n_ijk_range, particles); break;
    case C_MAKE_PHI_SUM: Reset_phi(phi); Reset_phi(phi_sum); Make_phi_particle_sum(phi, phi_sum, particles); break;
    case C_MAKE_U_SUM: Reset_u(up); Make_u_particle_sum(up, phi_sum, particles); break;
    case C_F_HYDRO: Calc_f_hydro_correct_precision(particles, phi_sum, u, jikan); break;
    case C_LJ:
      for (int n = 0; n < Particle_Number; n++)
        for (int d = 0; d < DIM; d++) particles[n].fr[d] = 0.0;
      Calc_f_Lennard_Jones(particles);
      break;
    case C_POS_EULER: MD_solver_position_Euler(particles, jikan); break;
    case C_POS_AB2: MD_solver_position_AB2(particles, jikan); break;
    case C_VEL_EULER: MD_solver_velocity_Euler(particles, jikan); break;
    case C_VEL_AB2: MD_solver_velocity_AB2_hydro(particles, jikan); break;
    case C_DIELECTRIC_FIELD:
      Make_dielectric_field(particles, epsilon, work_buf, eps_particle_top, eps_particle_bottom, eps_fluid);
      break;
    case C_BUILD_RHS: Build_rhs(work_buf, rho_free_buf, epsilon, E_ext); break;
    case C_SOLVE_POTENTIAL:
      Charge_field2potential_dielectric(rho_free_buf, Potential, epsilon, work_buf, E_ext);
      break;
    case C_MAXWELL:
      Make_Maxwell_force_x_on_fluid(f_particle, particles, Concentration, rho_free_buf, Potential, epsilon,
                                    grad_epsilon, jikan);
      break;
    case C_NSSOLUTE_EULER:
      NSsolute_solver_Euler(zeta, jikan, uk_dc, Concentration, particles, ijk_range, n_ijk_range);
      break;
    case C_SURFACE_NORMAL: Make_surface_normal(Surface_normal, particles); break;
    case C_F_PARTICLE_SOLE: Make_f_particle_dt_sole(f_particle, u, up, phi); break;
    case C_TRUNCATE: Truncate_two_third_rule(zeta[0]); Truncate_two_third_rule(zeta[1]); break;
    case C_CHARGE_FIELD:
      /* rho_free from the concentrations and the compact-sine profile in work;
       * with surface charges Conc_k2charge_field (work receives the Phi sum) */
      if (have_surface_charge) Conc_k2charge_field(particles, Concentration, rho_free_buf, work_buf, up[0]);
      else Conc_k2charge_field_no_surfase_charge(particles, Concentration, rho_free_buf, work_buf, up[0]);
      break;
    case C_INIT_ION: Init_rho_ion_dielectric(Concentration, particles, jikan); break;
    case C_CHARGE_OUTPUT: charge_output(); break;
    default: return 1;
  }
  return 0;
}

/* The reference's AVS writers on caller fields: Set_avs_parameters, Init_avs
 * and Init_avs_p (avs_output.cxx:46-186, avs_output_p.cxx:13-27), then one
 * frame: Output_avs_charge with fields[0..6] = u0 u1 u2 phi surface_charge
 * solute_charge potential ([NX][NY][NZ_]) and Output_avs_p of the harness
 * particles, at the harness ts and time (sp_3d_ns.cxx:482-497). */
int kref_avs(const char *dir, const char *name, int ascii, int num_snap, const double *const *fields) {
  snprintf(Out_dir, sizeof(Out_dir), "%s", dir);
  snprintf(Out_name, sizeof(Out_name), "%s", name);
  SW_OUTFORMAT = ascii ? OUT_AVS_ASCII : OUT_AVS_BINARY;
  Num_snap = num_snap;
  Set_avs_parameters(Avs_parameters);
  Init_avs(Avs_parameters);
  if (Particle_Number > 0) Init_avs_p(Avs_parameters);
  double *uf[DIM] = {(double *)fields[0], (double *)fields[1], (double *)fields[2]};
  Output_avs_charge(Avs_parameters, uf, (double *)fields[3], (double *)fields[4], (double *)fields[5],
                    (double *)fields[6], jikan);
  if (Particle_Number > 0) Output_avs_p(Avs_parameters, particles, jikan);
  return 0;
}

/* A x on unpadded length-N vectors (operate_dielectric.cxx:485-522). */
void kref_apply_A(const double *x, double *y) { Ax(x, y); }

}  // extern "C"
