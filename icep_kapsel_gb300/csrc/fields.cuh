// fields.cuh -- pointwise and stencil kernels on grid fields (k-space and
// real space). Each launcher names the reference routine it implements.
#pragma once
#include "common.cuh"

namespace icep {

// ---- k-space (one thread per complex mode) -------------------------------
// Truncate_two_third_rule_ooura (fft_wrapper.h:797-839)
template <typename R> void truncate_23(const Grid &g, const FieldBatch<R> &fb, cudaStream_t s);
// Zeta_k2u_k (fft_wrapper.cxx:614-711); uk_dc: device double[3]
template <typename R> void zeta_k2u_k(const Grid &g, const R *z0, const R *z1, const double *uk_dc, R *u0, R *u1, R *u2, cudaStream_t s);
// Truncate_two_third_rule of zeta (in place) then Zeta_k2u_k, one pass
template <typename R> void zeta_k2u_trunc(const Grid &g, R *z0, R *z1, const double *uk_dc, R *u0, R *u1, R *u2, cudaStream_t s);
// U_k2zeta_k (fft_wrapper.cxx:428-497); writes uk_dc (device double[3])
template <typename R> void u_k2zeta_k(const Grid &g, const R *u0, const R *u1, const R *u2, R *z0, R *z1, double *uk_dc, cudaStream_t s);
// The end of the step on spectra, one pass: u += P T f with T the 2/3
// truncation and P the solenoidal projection (the k-space part of
// Make_f_particle_dt_sole and Add_f_particle, f_particle.h:67-95), then
// U_k2zeta_k of the sum; f and u are spectra, u keeps the sum's spectrum
template <typename R> void sole_add_zeta(const Grid &g, R *const *f, R *const *u, R *z0, R *z1, double *uk_dc, cudaStream_t s);
// k-space half of U2advection_k (operate_omega.cxx:61-96) + Omega_k2zeta_k (fft_wrapper.cxx:248-284)
template <typename R> void advection_combine(const Grid &g, R *u0, R *u1, R *u2, R *a0, R *a1, cudaStream_t s);
// NS_solver_slavedEuler update (fluid_solver.cxx:345-365)
template <typename R> void ns_slaved_update(const Grid &g, R *z0, R *z1, const R *a0, const R *a1, double nu, double dt, cudaStream_t s);
// Truncate_two_third_rule of each component then Solenoidal_uk
// (operate_omega.cxx:187-220): the k-space part of Solenoidal_u
// (operate_omega.h:109-116), one pass
template <typename R> void truncate_solenoidal_uk(const Grid &g, R *u0, R *u1, R *u2, cudaStream_t s);
// A_k2da_k (fft_wrapper.cxx:214-237), optionally * Shift (Shift_vec_fw_imag,
// fft_wrapper.h:841-858), optionally minus e_ext*N at k = 0
// (Add_constant_field_k, fluid_solver.cxx:231-244; e_ext_n: a HOST array of
// the three values, or null); a may alias nothing.
template <typename R> void grad_k(const Grid &g, const R *a, R *d0, R *d1, R *d2, R scale, bool shift, const double *e_ext_n, cudaStream_t s);
// Truncate_two_third_rule of a (in place), d = scale i k a (unshifted) and
// cp = a, one pass (each species' diffusion flux, fluid_solver.cxx:246-292)
template <typename R> void grad_trunc_copy(const Grid &g, R *a, R *d0, R *d1, R *d2, R *cp, R scale, cudaStream_t s);
// U_k2divergence_k (fft_wrapper.cxx:896-920) / U_k2divergence_k_shift (fft_wrapper.h:879-900)
template <typename R> void div_k(const Grid &g, const R *u0, const R *u1, const R *u2, R *div, bool shift, cudaStream_t s);
// Add_zeta_viscous_term + Field_solver_Euler over the 2/3 region
// (operate_omega.cxx:170-185, fluid_solver.cxx:121-137) for zeta and c
template <typename R> void euler_update(const Grid &g, R *z0, R *z1, R *r0, R *r1, R *c0, R *c1, const R *cr0, const R *cr1, double nu, double dt, cudaStream_t s);
// Spectral inverse of the constant-permittivity staggered operator:
// a(k) *= -1 / (eps_ref |k|^2), a(0) = 0 (preconditioner of the SPECTRAL solver)
template <typename R> void inv_laplace_k(const Grid &g, R *a, double eps_ref, cudaStream_t s);
// y = a * x over all NX*NY*NZ_ values
template <typename R> void scale_copy(const Grid &g, const R *x, R *y, R a, cudaStream_t s);

// ---- real space (one thread per grid point, k < NZ) -----------------------
// real-space half of U2advection_k (operate_omega.cxx:31-45)
template <typename R> void advection_products(const Grid &g, R *u0, R *u1, R *u2, R *a0, R *a1, cudaStream_t s);
// phi = min(phi_sum, 1) (make_phi.cxx:262-273)
template <typename R> void phi_clip(const Grid &g, const R *phs, R *phi, cudaStream_t s);
// f = up - phi u (Make_f_particle_dt_nonsole, f_particle.h:37-60)
template <typename R> void f_nonsole(const Grid &g, R *const *f, R *const *up, const R *phi, R *const *u, cudaStream_t s);
// eps = ef*dc + (ep - ef)*dc*phi_sin, or eps = ef*dc + dc*eps_w (per particle)
// (Make_dielectric_field, operate_dielectric.cxx:298-307)
template <typename R> void eps_from_profile(const Grid &g, R *eps, const R *phi_sin, const R *eps_w, double ef, double ep, double dc, cudaStream_t s);
// Janus: eps = eps_j + eps_f (1 - phi_sin) Dc, eps_j the scattered particle
// term (operate_dielectric.cxx:276-292)
template <typename R> void eps_janus(const Grid &g, R *eps, const R *phi_sin, const R *eps_j, double ef, double dc, cudaStream_t s);
// rho += ze c (1 - phi) (Conc_k2charge_field_no_surfase_charge, operate_dielectric.cxx:135-160)
template <typename R> void charge_add(const Grid &g, R *rho, const R *c, const R *phi, double ze, bool first, cudaStream_t s);
// both species at once: rho (= or +=) ze0 c0 (1 - phi) then + ze1 c1 (1 - phi)
template <typename R> void charge_add2(const Grid &g, R *rho, const R *c0, const R *c1, const R *phi, double ze0, double ze1, bool first, cudaStream_t s);
// out = (ze0 c0 + ze1 c1) (1 - phi) (real points): the solute charge of the field output
template <typename R>
void solute_charge(const Grid &g, R *out, const R *c0, const R *c1, const R *phi, double ze0, double ze1, cudaStream_t s);
// w_d *= 0.5 (eps(i+e_d) + eps(i)) (Ax, operate_dielectric.cxx:494-510)
template <typename R> void eps_face_mul(const Grid &g, R *w0, R *w1, R *w2, const R *eps, cudaStream_t s);
// w_d = (0.5 eps(i+e_d) + 0.5 eps(i)) E_d (Interpolate_scalar_on_staggered_grid, operate_dielectric.cxx:57-76)
template <typename R> void eps_face_E(const Grid &g, R *w0, R *w1, R *w2, const R *eps, double e0, double e1, double e2, cudaStream_t s);
// y = a*x + b*y on real points
template <typename R> void axpby_real(const Grid &g, const R *x, R *y, R a, R b, cudaStream_t s);
// out_d(i) = 0.5 in_d(i) + 0.5 in_d(i - e_d) (Interpolate_vec_on_normal_grid, operate_dielectric.cxx:32-55)
template <typename R> void interp_normal(const Grid &g, R *const *out, R *const *in, cudaStream_t s);
// the same interpolation of in, written to out and out2 and added as
// acc += a * result (null targets skipped): the Maxwell force's copies and
// its Euler step u += dt/rho f (sp_3d_ns.cxx:83-94) in one pass
template <typename R> void interp_normal_to(const Grid &g, R *const *in, R *const *out, R *const *out2, R *const *acc, R a, cudaStream_t s);
// Maxwell stress terms (operate_dielectric.cxx:670-762)
template <typename R> void maxwell_e2(const Grid &g, const R *f0, const R *f1, const R *f2, R *w1, double e0, double e1, double e2, int ext, cudaStream_t s);
// out = face force from the staggered potential gradient grad_pot, the face
// charge and |E|^2 and the staggered permittivity gradient ge
template <typename R> void maxwell_face(const Grid &g, R *const *grad_pot, R *const *out, const R *rho, const R *w1, R *const *ge, double e0, double e1, double e2, int ext, cudaStream_t s);
// Nernst-Planck flux of one species in place: flux (the diffusion flux) + L_ze c gp, its
// component along the surface normal sn removed where sn != 0, then - c u
// when u is given (solute_rhs.cxx:150-210, 42-97)
template <typename R> void np_flux(const Grid &g, R *const *flux, const R *c, R *const *gp, double L_ze, R *const *sn, R *const *u, cudaStream_t s);
// real-space fill (k < NZ) of a constant
template <typename R> void fill_real(const Grid &g, R *a, R v, cudaStream_t s);
// The per-point terms of the free energy of Calc_free_energy_PB's Dielectric
// branch (operate_electrolyte.cxx:302-421) from the real densities c0, c1:
// ideal = sum_n (1 - phi) c_n (log c_n - 1); charge += sum_n ze_n c_n (1 - phi)
// (in place, species 0 first, as the reference accumulates); es = charge
// (pot/2 - E.r dx) with E = e (0 when ext is 0).
template <typename R>
void pb_energy_terms(const Grid &g, const R *c0, const R *c1, const R *phi, R *charge, const R *pot, double ze0,
                     double ze1, const double *e, double dx, int ext, R *ideal, R *es, cudaStream_t s);

}  // namespace icep
