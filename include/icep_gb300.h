/*
 * icep_gb300.h -- C-ABI of the GB300 (sm_103a) implementation of the
 * KAPSEL-ICEP per-timestep hot path.
 *
 * One context = one simulation on one GPU, one CUDA stream. All grid fields
 * and the particle array live in device memory for the lifetime of the
 * context; the host exchanges them in the reference's own layout
 * ([NX][NY][NZ_] doubles, icep_types.h). Every call returns 0 on success and
 * a positive status on failure (ICEP_ERR_*); no call exits the process and no
 * device code traps (reference: fatal errors call exit(EXIT_FAILURE),
 * macro.h:206-208).
 *
 * The reference seam each entry point replaces is cited as file:line of the
 * reference project (Takuma6/icep_kapsel).
 */
#ifndef ICEP_GB300_H
#define ICEP_GB300_H

#include <stddef.h>

#include "icep_types.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ICEP_OK 0
#define ICEP_ERR_ARG 1
#define ICEP_ERR_CUDA 2
#define ICEP_ERR_UNSUPPORTED 3
#define ICEP_ERR_NOT_CONVERGED 4
#define ICEP_ERR_STATE 5
#define ICEP_ERR_IO 6
/* A bounded wait inside a kernel ran out (an asynchronous copy or tensor-core
 * operation did not complete in time): the kernel skipped its work and
 * returned, the context stays usable, the step's results are not valid. */
#define ICEP_ERR_TIMEOUT 7

typedef struct icep_ctx icep_ctx;

/* Field identifiers for icep_get_field / icep_set_field. */
enum icep_field {
  ICEP_F_ZETA0 = 0, ICEP_F_ZETA1, ICEP_F_U0, ICEP_F_U1, ICEP_F_U2,
  ICEP_F_UP0, ICEP_F_UP1, ICEP_F_UP2, ICEP_F_PHI, ICEP_F_PHI_SUM,
  ICEP_F_F0, ICEP_F_F1, ICEP_F_F2, ICEP_F_POTENTIAL, ICEP_F_EPSILON,
  ICEP_F_GRAD_EPS0, ICEP_F_GRAD_EPS1, ICEP_F_GRAD_EPS2, ICEP_F_CONC0, ICEP_F_CONC1,
  ICEP_F_RHO_FREE, ICEP_F_WORK, ICEP_F_SURFACE_NORMAL0, ICEP_F_SURFACE_NORMAL1,
  ICEP_F_SURFACE_NORMAL2
};

/*
 * Context setup. Replaces the parameter derivation and allocation of
 * Set_global_parameters (input.cxx:286-440), Init_fft (fft_wrapper.cxx:166-199),
 * Mem_alloc_var (sp_3d_ns.cxx:295-340) and the stencil of Particle_domain
 * (profile.cxx:25-74). particles: n_particles entries, copied to the device.
 */
icep_ctx *icep_create(const icep_params *params, const icep_particle *particles, int n_particles, int *status);
void icep_destroy(icep_ctx *ctx);
/* Human-readable text of the last error of this context. */
const char *icep_last_error(const icep_ctx *ctx);

/*
 * main()'s initialisation after Init_Particle (sp_3d_ns.cxx:425-457): fluid
 * at rest with the rigidity force applied, and for Electrolyte +
 * Dielectric_property ON the uniform salt (Init_rho_ion_dielectric,
 * operate_electrolyte.cxx:912-979) and the first Poisson solve
 * (Init_potential_dielectric, operate_dielectric.cxx:574-609).
 */
int icep_init_state(icep_ctx *ctx);

/*
 * nsteps of the time loop body (sp_3d_ns.cxx:524-525): Time_evolution_hydro
 * (sp_3d_ns.cxx:24-186), the function the reference calls through the
 * pointer Time_evolution (sp_3d_ns.cxx:10), then jikan.time += dt.
 * A Poisson solve that meets a non-finite right-hand side or residual stops
 * the step with ICEP_ERR_NOT_CONVERGED (the reference keeps going); reaching
 * MaxIter is not an error, as in the reference (retry from a zero guess,
 * operate_dielectric.cxx:563-570).
 */
int icep_step(icep_ctx *ctx, int nsteps);

/*
 * Drop-in form of one call of Time_evolution (sp_3d_ns.cxx:10) on host
 * arrays: zeta (2 fields), uk_dc[3], conc (2 k-space fields, Electrolyte
 * only, may be NULL; a salt-free run has one, conc1 NULL), potential (1 real
 * field, Dielectric only, may be NULL)
 * and the particle array are uploaded, nsteps steps run on the GPU, and the
 * same arrays are written back.
 */
int icep_time_evolution(icep_ctx *ctx, double *zeta0, double *zeta1, double *uk_dc, double *conc0, double *conc1,
                        double *potential, icep_particle *particles, int nsteps);

/* Field and particle exchange in the reference layout (host pointers). */
int icep_get_field(icep_ctx *ctx, int field, double *host);
int icep_set_field(icep_ctx *ctx, int field, const double *host);
int icep_get_particles(icep_ctx *ctx, icep_particle *host);
int icep_set_particles(icep_ctx *ctx, const icep_particle *host);
int icep_get_uk_dc(icep_ctx *ctx, double *uk_dc);
int icep_set_uk_dc(icep_ctx *ctx, const double *uk_dc);
int icep_get_time(icep_ctx *ctx, int *ts, double *time);
int icep_set_time(icep_ctx *ctx, int ts, double time);
/* Checkpoint / restart (replaces Save_Restart_udf, resume.cxx:10-78, and
 * Force_restore_parameters, resume.cxx:308-398, with a binary file instead of
 * the UDF "resume" record). Saved: zeta, uk_dc, the particle array, ts and
 * time as in the reference, plus for electrolytes the concentrations' spectra
 * and the potential (and, in MIXED precision, the potential's float-float
 * spectrum and the previous one that the next solve extrapolates from), so
 * that a restarted run continues as the uninterrupted one. The load checks
 * mesh, particle count, precision and model against the context and leaves
 * the context unchanged when the file does not match (ICEP_ERR_ARG) or is
 * unreadable or truncated (ICEP_ERR_IO). */
int icep_save_checkpoint(icep_ctx *ctx, const char *path);

/* ---- input front end (no GPU needed) ------------------------------------- */
/* Reads a kapsel input UDF file (and the definitions it \include's) as the
 * reference's Gourmet_file_io (input.cxx:457-2139) does for the keys of this
 * path, with Set_global_parameters' auto time step (input.cxx:333-398), and
 * builds the initial particles as Init_Particle (init_particle.cxx:12-420):
 * uniform_random (glibc rand() sequence seeded with 10, kept private) or
 * user_specify positions; random, space_align or user orientations.
 * params gets precision FP64 and solver REF (the reference's arithmetic);
 * gts and num_snap are output.GTS and output.Num_snap (the run is
 * GTS * Num_snap steps). particles may be NULL to query n_particles; else it
 * needs max_particles >= n_particles. Returns ICEP_ERR_UNSUPPORTED (with the
 * reason in err) for settings outside this path: shear flows, chains and
 * rigid bodies, Dielectric_property OFF, pinned particles, lattice or random-walk
 * initial configurations, resumed runs (use icep_load_checkpoint). */
int icep_udf_read(const char *path, icep_params *params, icep_particle *particles, int max_particles,
                  int *n_particles, int *gts, int *num_snap, char *err, int err_len);
/* The text of one value of a UDF file by its dotted path, as the reference's
 * Location names it ("mesh.NPX",
 * "object_type.spherical_particle.Particle_spec[0].MASS_RATIO"; "<array>.size"
 * gives a list's length). On an error, value holds the message. */
int icep_udf_value(const char *path, const char *key, char *value, int len);
int icep_load_checkpoint(icep_ctx *ctx, const char *path);

/* Field output. The fields Output_dielectric_charge_field_data computes
 * (output.cxx:262-320) with velocity, phi and charge printed (what AVS
 * output prints, Init_output, output.cxx:18-22), as host FP64 arrays in the
 * reference layout [NX][NY][NZ_]; any pointer may be NULL:
 *   u0, u1, u2       Zeta_k2u(zeta, uk_dc)                            (u)
 *   phi              the sum of Phi over the particles, unclipped
 *                    (Make_phi_qq_particle, operate_electrolyte.cxx:179-243)
 *   surface_charge   its rescaled surface charge times 4 pi a^2       (up[0])
 *   solute_charge    e sum_n z_n c_n (1 - phi)                          (up[1])
 *   potential        the potential                                     (Potential)
 *   epsilon          the permittivity of the last step                 (up[2])
 * With no charged particle the surface charge is 0/0 = NaN everywhere, as the
 * reference's. The step state is left as it is (the reference transforms the
 * concentrations to real space and back). Electrolyte contexts only
 * (ICEP_ERR_UNSUPPORTED otherwise). */
int icep_charge_field_data(icep_ctx *ctx, double *u0, double *u1, double *u2, double *phi, double *surface_charge,
                           double *solute_charge, double *potential, double *epsilon);

/* AVS/Express output of the reference's default writers (SW_OUTFORMAT
 * OUT_AVS_BINARY, ascii = 0, or OUT_AVS_ASCII, ascii = 1), the same files,
 * names and bytes:
 *   icep_avs_init         Set_avs_parameters + Init_avs + Init_avs_p
 *                         (avs_output.cxx:46-186, avs_output_p.cxx:13-27):
 *                         out_dir/avs/, out_dir/<name>.fld (veclen 7, nstep),
 *                         out_dir/<name>.cod (uniform field extents, dx) and,
 *                         with particles, out_dir/<name>p.fld;
 *   icep_avs_charge_frame Output_avs_charge (avs_output.cxx:332-380): appends
 *                         the frame to <name>.fld and writes
 *                         out_dir/avs/<name>_<ts>.dat with the 7 fields
 *                         ux uy uz phi surface_charge rho e_potential as
 *                         float32, x fastest (fields[0..6], [NX][NY][NZ_]);
 *   icep_avs_particles    Output_avs_p (avs_output_p.cxx:73-157): appends to
 *                         <name>p.fld, writes avs/<name>p_<ts>.cod (z, y, x)
 *                         and .dat (radius, body axes from the quaternion);
 *   icep_output_avs       one frame of a context's current state (the field
 *                         frame, then the particle frame when there are
 *                         particles) at its ts and time, as the reference's
 *                         main loop writes every GTS steps (sp_3d_ns.cxx:482-497).
 * ICEP_ERR_IO when a file cannot be written. */
int icep_avs_init(const char *out_dir, const char *out_name, int ascii, int nx, int ny, int nz, double dx, int nstep,
                  int n_particles);
int icep_avs_charge_frame(const char *out_dir, const char *out_name, int ascii, int nx, int ny, int nz, int ts,
                          double time, const double *const *fields);
int icep_avs_particles(const char *out_dir, const char *out_name, int ascii, int ts, double time,
                       const icep_particle *particles, int n_particles, double radius);
int icep_output_avs(icep_ctx *ctx, const char *out_dir, const char *out_name, int ascii);

/* ---- phase entry points (operate on the context's device state) -------- */

/* A2a_k / A_k2a (fft_wrapper.h:681-723) in place on a host array of
 * NX*NY*NZ_ doubles. */
int icep_A2a_k(icep_ctx *ctx, double *a);
int icep_A_k2a(icep_ctx *ctx, double *a);

/* NS_solver_slavedEuler (fluid_solver.cxx:340-366) on ZETA0/1, uk_dc. */
int icep_NS_solver_slavedEuler(icep_ctx *ctx);
/* NSsolute_solver_Euler (fluid_solver.cxx:318-338), Dielectric branch. */
int icep_NSsolute_solver_Euler(icep_ctx *ctx);
/* Make_phi_particle_sum (make_phi.cxx:229-275, 519-523): PHI, PHI_SUM. */
int icep_Make_phi_particle_sum(icep_ctx *ctx);
/* Make_u_particle_sum (make_phi.cxx:329-370, 532-536): UP0..2 (zeroed first). */
int icep_Make_u_particle_sum(icep_ctx *ctx);
/* Make_surface_normal (make_phi.cxx:17-61): SURFACE_NORMAL0..2. */
int icep_Make_surface_normal(icep_ctx *ctx);
/* Calc_f_hydro_correct_precision (md_force.cxx:340-449) from U0..2, PHI_SUM. */
int icep_Calc_f_hydro_correct_precision(icep_ctx *ctx);
/* Calc_f_Lennard_Jones (md_force.h:81-84 -> md_force.cxx:16-171) into fr
 * (fr is cleared first). */
int icep_Calc_f_Lennard_Jones(icep_ctx *ctx);
/* The neighbour visits of the linked-cell scan: pairs (i, j), i > j, one
 * entry per visit. *n_pairs receives the total (may exceed max_pairs). */
int icep_lj_pairs(icep_ctx *ctx, int *pairs, int max_pairs, int *n_pairs);
/* Calc_f_Lennard_Jones on a caller-owned device array of n_particles
 * icep_particle (positions x in [0, L)), allocating nothing: no counterpart
 * in the reference, whose force routine (md_force.cxx:16-171) runs on host
 * arrays. Needs no context: the Lennard-Jones constants come from params
 * (mesh, DX, A, LJ_epsilon, LJ_powers, LJ_truncate) and fr of every particle
 * is overwritten with its Lennard-Jones force, the same values
 * icep_Calc_f_Lennard_Jones gives. For callers that hold their particles in
 * their own device memory and may not allocate during a step (a fixed device
 * memory budget, or no device-wide synchronisation from cudaMalloc/cudaFree
 * allowed mid-step). Work is queued on stream (cudaStream_t as void*; NULL:
 * the default stream) and the call does not wait for it.
 * Cell-list scratch is one fixed device array per device, shared by every
 * call: calls that may overlap in time race on it and must be serialised by
 * the caller. The first call on each device looks the array up
 * (cudaGetSymbolAddress, which may initialise the CUDA runtime); make that
 * first call before any stream capture. At most
 * ICEP_LJ_NOALLOC_MAX_PARTICLES particles and meshes up to 256^3; larger
 * inputs return ICEP_ERR_UNSUPPORTED with a message on stderr. */
#define ICEP_LJ_NOALLOC_MAX_PARTICLES 65536
int icep_Calc_f_Lennard_Jones_noalloc(const icep_params *params, icep_particle *d_particles, int n_particles,
                                      void *stream);
/* MD_solver_position_Euler/_AB2 (particle_solver.cxx:39-91) */
int icep_MD_solver_position(icep_ctx *ctx, int ab2);
/* MD_solver_velocity_Euler/_AB2_hydro (particle_solver.cxx:109-150, 252-295) */
int icep_MD_solver_velocity(icep_ctx *ctx, int ab2);
/* Make_dielectric_field (operate_dielectric.cxx:270-309): EPSILON, phi_sin in WORK. */
int icep_Make_dielectric_field(icep_ctx *ctx);
/* Conc_k2charge_field_no_surfase_charge (operate_dielectric.cxx:135-160):
 * RHO_FREE from CONC0/1 and the profile in WORK. */
int icep_Conc_k2charge_field(icep_ctx *ctx);
/* Build_rhs (operate_dielectric.cxx:524-540): WORK from EPSILON, RHO_FREE. */
int icep_Build_rhs(icep_ctx *ctx);
/* Ax (operate_dielectric.cxx:485-522) with the context's EPSILON, on
 * unpadded host vectors of NX*NY*NZ doubles (the MatrixReplacement matvec,
 * LinearOperator.h:70-82). */
int icep_Ax(icep_ctx *ctx, const double *x, double *ax);
/*
 * Charge_field2potential_dielectric (operate_dielectric.cxx:18-22, bound to
 * _LO at :592): POTENTIAL from RHO_FREE and EPSILON with the context's solver
 * (params.solver). iterations / error receive the statistics of the last
 * solve (error: recursive residual for REF, true relative residual for
 * SPECTRAL).
 */
int icep_Charge_field2potential_dielectric(icep_ctx *ctx, int *iterations, double *error);
/* Make_Maxwell_force_x_on_fluid (operate_dielectric.cxx:611-764): F0..2. */
int icep_Make_Maxwell_force_x_on_fluid(icep_ctx *ctx);
/* Statistics of the last Poisson solve of the context. */
int icep_solver_stats(icep_ctx *ctx, int *iterations, double *error, long *matvecs);
/* Steps of the context taken as one CUDA graph so far (no reference
 * counterpart): with precision ICEP_MIXED, an electrolyte and the fused
 * Poisson passes, a step from the second on is captured once -- the Poisson
 * solve's refinement sweeps and iterations as device-side loops -- and
 * replayed, alone (icep_step) or with the other replicas of a batch
 * (icep_batch_step); ICEP_GRAPHS=0 at context creation turns this off. */
int icep_step_graphs(icep_ctx *ctx, long *n);
/* Generic phase dispatch (ids of the step's phases, numbered as in the
 * checker used by the tests). */
int icep_call(icep_ctx *ctx, int fn);

/* ---- batches of independent replicas (no reference counterpart) ---------
 * The reference runs one system per process; an ensemble there is many
 * processes. A batch holds n contexts (any mix of meshes, particle counts and
 * parameters), each with its own CUDA stream. icep_batch_step advances all
 * of them and returns when every replica has finished: once every replica
 * can take its step as a CUDA graph (MIXED electrolytes on the fused Poisson
 * passes, from their second step on), all replicas' steps are captured into
 * one graph -- independent branches, the Poisson solves' loops on the device
 * -- and each batch step is one graph launch and one host wait; otherwise the
 * replicas step from a pool of host threads, their kernels running
 * concurrently on their streams. */
typedef struct icep_batch icep_batch;
/* params[i], particles[i] (params[i].n_particles entries) for replica i. */
icep_batch *icep_batch_create(int n, const icep_params *params, const icep_particle *const *particles, int *status);
void icep_batch_destroy(icep_batch *batch);
int icep_batch_size(const icep_batch *batch);
/* The context of replica i, for the per-replica calls (get/set fields, ...). */
icep_ctx *icep_batch_context(icep_batch *batch, int i);
/* Text of the first error of the last batch call ("replica i: ..."). */
const char *icep_batch_last_error(const icep_batch *batch);
int icep_batch_init_state(icep_batch *batch);
int icep_batch_step(icep_batch *batch, int nsteps);

/* ---- learned Poisson preconditioner (no reference counterpart) -----------
 * Contexts created with precision ICEP_MIXED and solver ICEP_SOLVER_LEARNED
 * (cubic mesh 32..128) solve the inner correction systems of
 * Charge_field2potential_dielectric with flexible GMRES whose preconditioner
 * is the spectral one applied to the residual plus a U-Net correction of it
 * (computed on the half-resolution grid, BF16 tensor cores); the spectral BiCGSTAB is the fallback when the
 * flexible iteration stagnates, and the true residual (float-float, 48-bit)
 * decides convergence as for the plain solver. Before training (or with
 * icep_learned_enable(ctx, 0)) the network is not applied. */
/* Train on the GPU: `configs` random particle configurations (the context's
 * radius, new positions, a random direction of E_ext; with per-particle
 * permittivity on, eps_p uniform in [1, 10] and between a quarter of the
 * context's particle count and all of it present -- the others take the
 * fluid's permittivity), each for `steps_per_config` Adam steps along the
 * chain of residuals r -> r - A P(r) starting from the right-hand side; loss
 * |r - A P(r)|^2 / |r|^2 with P(r) = M^-1 (r + rms(r) prolong(net(eps, r))).
 * The context's particles and field are restored afterwards. The trained
 * parameters are kept only if they lower the one-step loss on the context's
 * own residuals (icep_learned_eval with chain 4, configurations not trained
 * on) below the spectral preconditioner's; otherwise the earlier parameters
 * come back and the network is not applied until icep_learned_enable(ctx, 1)
 * or a later training that is kept. */
int icep_learned_train(icep_ctx *ctx, int configs, int steps_per_config, unsigned seed, double lr, double *loss_first,
                       double *loss_last);
/* 1: apply the network in the preconditioner, 0: spectral part only. */
int icep_learned_enable(icep_ctx *ctx, int on);
/* Mean one-step loss |r - A P(r)|^2 / |r|^2 of the spectral-only and of the
 * learned preconditioner P on the same residuals: the context's current
 * right-hand side and the next chain-1 residuals of the spectral iteration. */
int icep_learned_eval(icep_ctx *ctx, int chain, double *loss_spectral, double *loss_learned);
/* Number of network parameters (FP32 master copy) and their exchange. */
long icep_learned_nparams(icep_ctx *ctx);
int icep_learned_get_params(icep_ctx *ctx, double *params);
int icep_learned_set_params(icep_ctx *ctx, const double *params);
/* The network alone, for checks: input from the fine-grid permittivity and
 * residual (real fields, reference layout), output y on the half-resolution
 * grid ((NX/2)^3 values, z fastest); the backward pass after it gives the
 * parameter gradient for dL/dy = gy. */
int icep_learned_forward(icep_ctx *ctx, const double *eps, const double *r, double eps_ref, double *y);
int icep_learned_backward(icep_ctx *ctx, const double *gy, double *grad);
/* Plain-solver fallbacks and preconditioner applications of the last solve. */
int icep_learned_stats(icep_ctx *ctx, int *fallbacks, int *precond_apps);

/* ---- measurement helpers (no reference counterpart) --------------------- */
/* Average device time of `reps` launches of one kernel group on the
 * context's stream (CUDA events): which 0..3 = one pass of the 3D FFT
 * (0: z rows + y pencils forward, 1: x pencils forward, 2: x pencils inverse,
 * 3: y pencils + z rows inverse), 7 = forward 3D FFT, 8 = inverse 3D FFT,
 * 9 = Ax, 10 = the MIXED solve's float-float true residual b^ - A x^ (a
 * MIXED context with an electrolyte, after a step). batch: fields per
 * launch (1..5). bytes: algorithmic bytes per launch (one field read and
 * written per transform or pass). */
int icep_time_kernel(icep_ctx *ctx, int which, int batch, int reps, double *ms, double *bytes);
/* icep_step with CUDA events recorded on the context's stream around it;
 * ms receives the device time of the nsteps steps. */
int icep_step_timed(icep_ctx *ctx, int nsteps, double *ms);
/* Device time accumulated per phase of the step when the context was
 * created with the environment variable ICEP_PHASE_PROFILE=1 (events at
 * phase boundaries): 0 fluid/solute update, 1 velocity + particle positions
 * + profile, 2 hydrodynamic force + permittivity + free charge, 3 Poisson
 * solve, 4 Maxwell stress, 5 Maxwell force on the fluid + projection,
 * 6 particle forces and velocities, 7 particle velocity field, 8 rigidity
 * force and back to vorticity, 9 unused. Returns ICEP_ERR_STATE when
 * profiling is off. */
int icep_phase_times(icep_ctx *ctx, double *ms, int n);
/* The tile autotuner of the fused Poisson passes (no counterpart in the
 * reference): at context creation (MIXED electrolyte on a mesh the fused
 * passes cover) every candidate tile shape is timed on scratch fields and the
 * fastest kept, per mesh for the process (ICEP_AUTOTUNE=0 keeps the
 * defaults; ICEP_KOP_TILES="xinv,xfwd,plane" sets the picks, untimed).
 * picks[3] receives the x pencils per block of the inverse and forward x
 * passes and the plane pass's kernel (0 register-resident, 1 shared-memory);
 * us[8] (optional) the measured times per launch: xinv 8/16/32, xfwd
 * 8/16/32, plane register/shared (0 for candidates the mesh lacks or picks
 * set by hand). ICEP_ERR_STATE for contexts without tuned passes. */
int icep_autotune_picks(icep_ctx *ctx, int *picks, double *us);
/* Check of the bounded device waits (no counterpart in the reference):
 * launches one kernel in a mode that issues no asynchronous copy or MMA, so
 * that its mbarrier wait runs out after ~50 us -- kernel 1: the fused plane
 * pass of the k-space Poisson operator (MIXED context, 64^3 or 128^3 class
 * meshes), 2: the network's tcgen05 convolution (solver LEARNED) -- and
 * returns the status a solve would return when that happens:
 * ICEP_ERR_TIMEOUT, with the context left usable (ICEP_ERR_UNSUPPORTED for
 * other contexts, ICEP_OK if the wait did not run out). */
int icep_selftest_wait(icep_ctx *ctx, int kernel);
/* Kernels launched by this library so far (all contexts). */
unsigned long long icep_kernel_launches(void);
/* Algorithmic bytes of the kernels launched so far (all contexts): every
 * launch adds its external inputs and outputs (grid fields read or written,
 * one field per field and pass of a 3D transform, scatter/gather stencil
 * traffic); a step's increase divided by its time is its roofline figure. */
unsigned long long icep_algorithmic_bytes(void);
/* Page-lock / release a caller's host buffer for the drop-in transfers. The
 * buffer is registered as mapped: icep_time_evolution and the field getters
 * and setters then read and write it from their conversion kernels over the
 * CPU-GPU link, with no staging copy. Release it only when no call that uses
 * it is running. */
int icep_pin_host(void *ptr, size_t bytes);
int icep_unpin_host(void *ptr);

/* Stream of the context (cudaStream_t as void*), for callers that order
 * their own device work after the library's. */
void *icep_stream(icep_ctx *ctx);
/* Block until the context's queued work has finished. */
int icep_synchronize(icep_ctx *ctx);

/* Measurement hook (no counterpart in the reference): time every launch of
 * one kernel class with CUDA events on its stream until icep_probe_stop.
 * kind: 1 fused plane pass of the k-space Poisson operator, 2 its fused
 * inverse x pass, 3 its fused forward x pass. At most max_launches launches
 * are timed. Process-wide; not for concurrent use. */
int icep_probe_start(int kind, int max_launches);
/* Ends the probe: total device time (ms), launches timed and their total
 * algorithmic bytes (the kernel's external inputs and outputs). */
int icep_probe_stop(double *ms_total, long long *launches_timed, double *bytes_total);

#ifdef __cplusplus
}
#endif
#endif
