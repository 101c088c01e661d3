// engine.cuh -- one simulation context on the GPU: device state, the step
// sequence of Time_evolution_hydro (sp_3d_ns.cxx:24-186) and its phases.
#pragma once
#include <string>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "particles.cuh"

namespace icep {

struct EngineBase {
  virtual ~EngineBase() {}
  std::string err;
  virtual int init_state() = 0;
  virtual int step(int n) = 0;
  virtual int get_field(int id, double *host) = 0;
  virtual int set_field(int id, const double *host) = 0;
  // n fields at once (the drop-in call's host I/O): all copies queued, one
  // synchronisation; host arrays should be pinned for the copies to overlap
  virtual int set_fields(const int *ids, const double *const *host, int n) = 0;
  virtual int get_fields(const int *ids, double *const *host, int n) = 0;
  virtual int get_particles(icep_particle *h) = 0;
  virtual int set_particles(const icep_particle *h) = 0;
  virtual int get_uk_dc(double *v) = 0;
  virtual int set_uk_dc(const double *v) = 0;
  // The drop-in call (icep_time_evolution): uk_dc, the particles and the n
  // fields up, nsteps steps, the same back into the same host arrays, with
  // the copies queued and the stream synchronised only where the host needs
  // a result (the potential's comparison, the steps' solver status, the end)
  virtual int time_evolution_host(const int *ids, double *const *host, int n, double *uk_dc,
                                  icep_particle *parts, int nsteps) = 0;
  virtual int fft_host(double *a, bool forward) = 0;
  virtual int call(int fn) = 0;
  virtual int apply_A_host(const double *x, double *y) = 0;
  virtual int lj_pairs(int *pairs, int max_pairs, int *n) = 0;
  virtual int sync() = 0;
  virtual cudaStream_t stream() const = 0;
  // Time `reps` back-to-back launches of one kernel group on the context's
  // stream with CUDA events: which = 0..3 one FFT pass (fft_pass), 7 = R2C,
  // 8 = C2R, 9 = Ax. ms: average per launch; bytes: algorithmic bytes moved
  // per launch (read + write of the fields touched, one field = N*sizeof).
  virtual int time_kernel(int which, int batch, int reps, double *ms, double *bytes) = 0;
  // accumulated device time per step phase (ICEP_PHASE_PROFILE=1 at create)
  virtual int phase_times(double *ms, int n) = 0;
  // checkpoint / restart of the step state (fields, particles, time)
  // Output_dielectric_charge_field_data's fields (u0 u1 u2 phi surface
  // solute potential eps) into host FP64 arrays; NULL entries are skipped
  virtual int charge_field_data(double *const *out) = 0;
  virtual const icep_params &params() const = 0;
  virtual int n_particles() const = 0;
  virtual int save_checkpoint(const char *path) = 0;
  virtual int load_checkpoint(const char *path) = 0;
  // learned preconditioner (MIXED precision with solver ICEP_SOLVER_LEARNED)
  virtual int learned_train(int configs, int steps, unsigned seed, double lr, double *loss_first, double *loss_last) {
    return unsupported_learned();
  }
  virtual int learned_enable(int on) { return unsupported_learned(); }
  virtual int learned_eval(int chain, double *loss_spectral, double *loss_learned) { return unsupported_learned(); }
  virtual long learned_nparams() { return 0; }
  virtual int learned_params(double *buf, bool get) { return unsupported_learned(); }
  virtual int learned_forward(const double *eps, const double *r, double eps_ref, double *y) {
    return unsupported_learned();
  }
  virtual int learned_backward(const double *gy, double *grad) { return unsupported_learned(); }
  // the tile autotuner's picks for the fused Poisson passes (see kop.cuh)
  virtual int tile_picks(int *picks, double *us) {
    err = "no tuned fused passes in this context";
    return ICEP_ERR_STATE;
  }
  // launch one kernel whose bounded wait must run out (1: fused plane pass,
  // 2: tcgen05 convolution) and return the status a solve would return
  virtual int selftest_wait(int kernel) {
    err = "the wait self-test needs a MIXED context (kernel 1) or solver LEARNED (kernel 2)";
    return ICEP_ERR_UNSUPPORTED;
  }
  // The step as one CUDA graph (MIXED electrolytes on the fused passes):
  // whether the next step can run so; its capture appended to a graph after
  // the given nodes (which receive its last nodes); and, after a replay has
  // finished, the solve's status read back (advance: time and step count
  // advanced as step() does). A batch captures all its replicas into one
  // graph.
  virtual bool whole_step_ok() const { return false; }
  virtual int capture_step(cudaGraph_t gr, std::vector<cudaGraphNode_t> &deps) {
    err = "no step graph for this context";
    return ICEP_ERR_UNSUPPORTED;
  }
  virtual int step_graph_done(bool advance) { return ICEP_ERR_UNSUPPORTED; }
  long graph_steps = 0;  // steps run as one graph (alone or in a batch graph)
  // E_ext at the context's current time (an AC field's phase)
  virtual void refresh_field() {}
  int unsupported_learned() {
    err = "the learned preconditioner needs precision MIXED and solver LEARNED";
    return ICEP_ERR_UNSUPPORTED;
  }
  int last_fallbacks = 0;      // plain-solver fallbacks of the last learned solve
  int last_precond_apps = 0;   // preconditioner applications of the last learned solve
  int ts = 0;
  double time = 0.0;
  int last_iters = 0;
  double last_error = 0.0;
  long matvecs = 0;
};

EngineBase *make_engine(const icep_params &p, const icep_particle *parts, int np, int *status, std::string &err);
// The device address of host memory [p, p + bytes) when it lies inside one
// range pinned (mapped) through icep_pin_host, else nullptr.
void *host_mapped(const void *p, size_t bytes);

// ids of Engine::call (same numbering as the oracle's ko_call)
enum CallId {
  C_ZETA_K2U_K = 1, C_U_K2ZETA_K, C_U2ADVECTION_K, C_SOLENOIDAL_U, C_NS_SLAVED_EULER,
  C_MAKE_PHI_SUM, C_MAKE_U_SUM, C_F_HYDRO, C_LJ, C_POS_EULER, C_POS_AB2, C_VEL_EULER,
  C_VEL_AB2, C_DIELECTRIC_FIELD, C_BUILD_RHS, C_SOLVE_POTENTIAL, C_MAXWELL, C_NSSOLUTE_EULER,
  C_SURFACE_NORMAL, C_F_PARTICLE_SOLE, C_TRUNCATE, C_CHARGE_FIELD, C_INIT_ION, C_ZETA_K2U,
  // 25 is the checkers' field-output call; MIXED only (a check of the fused
  // operator): WORK = B WV1 = A M^-1 WV1 on the half spectrum in WV1, through
  // the three fused passes
  C_APPLY_BK = 26
};

}  // namespace icep
