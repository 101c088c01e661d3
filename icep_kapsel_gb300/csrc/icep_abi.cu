// icep_abi.cu -- the extern "C" entry points declared in include/icep_gb300.h.
#include <string.h>

#include <stdint.h>

#include <algorithm>
#include <mutex>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "../../include/icep_gb300.h"
#include "engine.cuh"

namespace icep {
unsigned long long g_kernel_launches = 0;
unsigned long long g_alg_bytes = 0;

// Host ranges pinned through icep_pin_host, registered as mapped: the
// drop-in calls read and write them from kernels over the CPU-GPU link.
namespace {
struct PinRange {
  uintptr_t lo;
  size_t n;
  char *dev;
};
std::mutex g_pin_mu;
std::vector<PinRange> g_pins;
}  // namespace
void *host_mapped(const void *p, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_pin_mu);
  const uintptr_t a = (uintptr_t)p;
  for (const PinRange &r : g_pins)
    if (a >= r.lo && bytes <= r.n && a - r.lo <= r.n - bytes) return r.dev + (a - r.lo);
  return nullptr;
}
}  // namespace icep

struct icep_ctx {
  icep::EngineBase *e = nullptr;
  std::string err;
};

namespace {
int wrap(icep_ctx *c, int st) {
  if (st != ICEP_OK && c && c->e) c->err = c->e->err;
  return st;
}
bool ok(icep_ctx *c) { return c && c->e; }
}  // namespace

extern "C" {

icep_ctx *icep_create(const icep_params *params, const icep_particle *particles, int n_particles, int *status) {
  if (!params || (n_particles > 0 && !particles)) {
    if (status) *status = ICEP_ERR_ARG;
    return nullptr;
  }
  std::string err;
  int st = ICEP_OK;
  icep::EngineBase *e = icep::make_engine(*params, particles, n_particles, &st, err);
  if (status) *status = st;
  if (!e) {
    fprintf(stderr, "icep_create: %s\n", err.c_str());
    return nullptr;
  }
  icep_ctx *c = new icep_ctx();
  c->e = e;
  return c;
}

void icep_destroy(icep_ctx *ctx) {
  if (!ctx) return;
  delete ctx->e;
  delete ctx;
}

const char *icep_last_error(const icep_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int icep_init_state(icep_ctx *c) { return ok(c) ? wrap(c, c->e->init_state()) : ICEP_ERR_ARG; }
int icep_step(icep_ctx *c, int n) {
  if (!ok(c) || n < 0) return ICEP_ERR_ARG;
  return wrap(c, c->e->step(n));
}

int icep_step_graphs(icep_ctx *c, long *n) {
  if (!ok(c) || !n) return ICEP_ERR_ARG;
  *n = c->e->graph_steps;
  return ICEP_OK;
}

int icep_get_field(icep_ctx *c, int field, double *host) {
  if (!ok(c) || !host) return ICEP_ERR_ARG;
  return wrap(c, c->e->get_field(field, host));
}
int icep_set_field(icep_ctx *c, int field, const double *host) {
  if (!ok(c) || !host) return ICEP_ERR_ARG;
  return wrap(c, c->e->set_field(field, host));
}
int icep_get_particles(icep_ctx *c, icep_particle *h) {
  if (!ok(c) || !h) return ICEP_ERR_ARG;
  return wrap(c, c->e->get_particles(h));
}
int icep_set_particles(icep_ctx *c, const icep_particle *h) {
  if (!ok(c) || !h) return ICEP_ERR_ARG;
  return wrap(c, c->e->set_particles(h));
}
int icep_get_uk_dc(icep_ctx *c, double *v) { return ok(c) && v ? wrap(c, c->e->get_uk_dc(v)) : ICEP_ERR_ARG; }
int icep_set_uk_dc(icep_ctx *c, const double *v) { return ok(c) && v ? wrap(c, c->e->set_uk_dc(v)) : ICEP_ERR_ARG; }
int icep_get_time(icep_ctx *c, int *ts, double *time) {
  if (!ok(c)) return ICEP_ERR_ARG;
  if (ts) *ts = c->e->ts;
  if (time) *time = c->e->time;
  return ICEP_OK;
}
int icep_set_time(icep_ctx *c, int ts, double time) {
  if (!ok(c)) return ICEP_ERR_ARG;
  c->e->ts = ts;
  c->e->time = time;
  return ICEP_OK;
}

int icep_save_checkpoint(icep_ctx *c, const char *path) {
  return ok(c) && path ? wrap(c, c->e->save_checkpoint(path)) : ICEP_ERR_ARG;
}
int icep_load_checkpoint(icep_ctx *c, const char *path) {
  return ok(c) && path ? wrap(c, c->e->load_checkpoint(path)) : ICEP_ERR_ARG;
}

int icep_charge_field_data(icep_ctx *c, double *u0, double *u1, double *u2, double *phi, double *surface_charge,
                           double *solute_charge, double *potential, double *epsilon) {
  if (!ok(c)) return ICEP_ERR_ARG;
  double *out[8] = {u0, u1, u2, phi, surface_charge, solute_charge, potential, epsilon};
  return wrap(c, c->e->charge_field_data(out));
}

int icep_output_avs(icep_ctx *c, const char *out_dir, const char *out_name, int ascii) {
  if (!ok(c) || !out_dir || !out_name) return ICEP_ERR_ARG;
  icep::EngineBase *e = c->e;
  const icep_params &p = e->params();
  const size_t nf = (size_t)p.nx * p.ny * (2 * (p.nz / 2 + 1));
  std::vector<double> buf(7 * nf);
  double *out[8];
  for (int k = 0; k < 7; k++) out[k] = buf.data() + k * nf;
  out[7] = nullptr;
  int st = e->charge_field_data(out);
  if (st) return wrap(c, st);
  const double *fields[7] = {out[0], out[1], out[2], out[3], out[4], out[5], out[6]};
  st = icep_avs_charge_frame(out_dir, out_name, ascii, p.nx, p.ny, p.nz, e->ts, e->time, fields);
  if (st) {
    c->err = "cannot write the AVS field frame";
    return st;
  }
  const int np = e->n_particles();
  if (np > 0) {
    std::vector<icep_particle> parts((size_t)np);
    if ((st = e->get_particles(parts.data()))) return wrap(c, st);
    st = icep_avs_particles(out_dir, out_name, ascii, e->ts, e->time, parts.data(), np, p.a * p.dx);
    if (st) c->err = "cannot write the AVS particle frame";
  }
  return st;
}

int icep_time_evolution(icep_ctx *c, double *zeta0, double *zeta1, double *uk_dc, double *conc0, double *conc1,
                        double *potential, icep_particle *particles, int nsteps) {
  if (!ok(c) || !zeta0 || !zeta1 || !uk_dc || !particles || nsteps < 0) return ICEP_ERR_ARG;
  icep::EngineBase *e = c->e;
  // the fields go as one batch each way, queued with uk_dc and the particles
  // (the stream synchronised where the host needs a result); a potential
  // passed back as this call returned it keeps the Poisson solver's state
  int ids[5] = {icep::F_ZETA0, icep::F_ZETA1};
  double *ptr[5] = {zeta0, zeta1};
  int n = 2;
  if (conc0) { ids[n] = icep::F_C0; ptr[n++] = conc0; }
  if (conc1) { ids[n] = icep::F_C1; ptr[n++] = conc1; }
  if (potential) { ids[n] = icep::F_POT; ptr[n++] = potential; }
  return wrap(c, e->time_evolution_host(ids, ptr, n, uk_dc, particles, nsteps));
}

int icep_A2a_k(icep_ctx *c, double *a) { return ok(c) && a ? wrap(c, c->e->fft_host(a, true)) : ICEP_ERR_ARG; }
int icep_A_k2a(icep_ctx *c, double *a) { return ok(c) && a ? wrap(c, c->e->fft_host(a, false)) : ICEP_ERR_ARG; }

int icep_NS_solver_slavedEuler(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_NS_SLAVED_EULER)) : ICEP_ERR_ARG; }
int icep_NSsolute_solver_Euler(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_NSSOLUTE_EULER)) : ICEP_ERR_ARG; }
int icep_Make_phi_particle_sum(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_MAKE_PHI_SUM)) : ICEP_ERR_ARG; }
int icep_Make_u_particle_sum(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_MAKE_U_SUM)) : ICEP_ERR_ARG; }
int icep_Make_surface_normal(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_SURFACE_NORMAL)) : ICEP_ERR_ARG; }
int icep_Calc_f_hydro_correct_precision(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_F_HYDRO)) : ICEP_ERR_ARG; }
int icep_Calc_f_Lennard_Jones(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_LJ)) : ICEP_ERR_ARG; }
int icep_lj_pairs(icep_ctx *c, int *pairs, int max_pairs, int *n_pairs) {
  if (!ok(c) || !n_pairs || (max_pairs > 0 && !pairs)) return ICEP_ERR_ARG;
  return wrap(c, c->e->lj_pairs(pairs, max_pairs, n_pairs));
}
int icep_MD_solver_position(icep_ctx *c, int ab2) {
  return ok(c) ? wrap(c, c->e->call(ab2 ? icep::C_POS_AB2 : icep::C_POS_EULER)) : ICEP_ERR_ARG;
}
int icep_MD_solver_velocity(icep_ctx *c, int ab2) {
  return ok(c) ? wrap(c, c->e->call(ab2 ? icep::C_VEL_AB2 : icep::C_VEL_EULER)) : ICEP_ERR_ARG;
}
int icep_Make_dielectric_field(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_DIELECTRIC_FIELD)) : ICEP_ERR_ARG; }
int icep_Conc_k2charge_field(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_CHARGE_FIELD)) : ICEP_ERR_ARG; }
int icep_Build_rhs(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_BUILD_RHS)) : ICEP_ERR_ARG; }
int icep_Ax(icep_ctx *c, const double *x, double *ax) {
  if (!ok(c) || !x || !ax) return ICEP_ERR_ARG;
  return wrap(c, c->e->apply_A_host(x, ax));
}
int icep_Charge_field2potential_dielectric(icep_ctx *c, int *iterations, double *error) {
  if (!ok(c)) return ICEP_ERR_ARG;
  int st = wrap(c, c->e->call(icep::C_SOLVE_POTENTIAL));
  if (iterations) *iterations = c->e->last_iters;
  if (error) *error = c->e->last_error;
  return st;
}
int icep_Make_Maxwell_force_x_on_fluid(icep_ctx *c) { return ok(c) ? wrap(c, c->e->call(icep::C_MAXWELL)) : ICEP_ERR_ARG; }
int icep_solver_stats(icep_ctx *c, int *iterations, double *error, long *matvecs) {
  if (!ok(c)) return ICEP_ERR_ARG;
  if (iterations) *iterations = c->e->last_iters;
  if (error) *error = c->e->last_error;
  if (matvecs) *matvecs = c->e->matvecs;
  return ICEP_OK;
}
void *icep_stream(icep_ctx *c) { return ok(c) ? (void *)c->e->stream() : nullptr; }
int icep_synchronize(icep_ctx *c) { return ok(c) ? wrap(c, c->e->sync()) : ICEP_ERR_ARG; }

int icep_time_kernel(icep_ctx *c, int which, int batch, int reps, double *ms, double *bytes) {
  if (!ok(c) || !ms || !bytes) return ICEP_ERR_ARG;
  return wrap(c, c->e->time_kernel(which, batch, reps, ms, bytes));
}
int icep_step_timed(icep_ctx *c, int nsteps, double *ms) {
  if (!ok(c) || nsteps < 0 || !ms) return ICEP_ERR_ARG;
  cudaStream_t s = c->e->stream();
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return ICEP_ERR_CUDA;
  cudaEventRecord(e0, s);
  int st = c->e->step(nsteps);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = (double)t;
  return wrap(c, st);
}
int icep_phase_times(icep_ctx *c, double *ms, int n) {
  if (!ok(c) || !ms) return ICEP_ERR_ARG;
  return wrap(c, c->e->phase_times(ms, n));
}
unsigned long long icep_kernel_launches(void) { return __atomic_load_n(&icep::g_kernel_launches, __ATOMIC_RELAXED); }
unsigned long long icep_algorithmic_bytes(void) { return __atomic_load_n(&icep::g_alg_bytes, __ATOMIC_RELAXED); }
int icep_pin_host(void *p, size_t bytes) {
  if (!p || !bytes) return ICEP_ERR_ARG;
  if (cudaHostRegister(p, bytes, cudaHostRegisterMapped) != cudaSuccess) {
    cudaGetLastError();  // reported here: not left for the context's next call to find
    return ICEP_ERR_CUDA;
  }
  void *dev = nullptr;
  if (cudaHostGetDevicePointer(&dev, p, 0) == cudaSuccess && dev) {
    std::lock_guard<std::mutex> lk(icep::g_pin_mu);
    icep::g_pins.push_back(icep::PinRange{(uintptr_t)p, bytes, (char *)dev});
  } else {
    cudaGetLastError();  // pinned, not mapped: the calls stage through device buffers
  }
  return ICEP_OK;
}
int icep_unpin_host(void *p) {
  if (!p) return ICEP_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(icep::g_pin_mu);
    for (size_t k = 0; k < icep::g_pins.size();)
      if (icep::g_pins[k].lo == (uintptr_t)p) icep::g_pins.erase(icep::g_pins.begin() + (long)k);
      else k++;
  }
  if (cudaHostUnregister(p) != cudaSuccess) {
    cudaGetLastError();
    return ICEP_ERR_CUDA;
  }
  return ICEP_OK;
}

int icep_autotune_picks(icep_ctx *c, int *picks, double *us) {
  return (ok(c) && picks) ? wrap(c, c->e->tile_picks(picks, us)) : ICEP_ERR_ARG;
}
int icep_selftest_wait(icep_ctx *c, int kernel) { return ok(c) ? wrap(c, c->e->selftest_wait(kernel)) : ICEP_ERR_ARG; }

/* generic dispatch used by the Python layer (same numbering as the oracle) */
int icep_call(icep_ctx *c, int fn) { return ok(c) ? wrap(c, c->e->call(fn)) : ICEP_ERR_ARG; }

/* learned preconditioner */
int icep_learned_train(icep_ctx *c, int configs, int steps_per_config, unsigned seed, double lr, double *loss_first,
                       double *loss_last) {
  return ok(c) ? wrap(c, c->e->learned_train(configs, steps_per_config, seed, lr, loss_first, loss_last)) : ICEP_ERR_ARG;
}
int icep_learned_enable(icep_ctx *c, int on) { return ok(c) ? wrap(c, c->e->learned_enable(on)) : ICEP_ERR_ARG; }
int icep_learned_eval(icep_ctx *c, int chain, double *loss_spectral, double *loss_learned) {
  return ok(c) && loss_spectral && loss_learned ? wrap(c, c->e->learned_eval(chain, loss_spectral, loss_learned))
                                                : ICEP_ERR_ARG;
}
long icep_learned_nparams(icep_ctx *c) { return ok(c) ? c->e->learned_nparams() : 0; }
int icep_learned_get_params(icep_ctx *c, double *params) {
  return ok(c) && params ? wrap(c, c->e->learned_params(params, true)) : ICEP_ERR_ARG;
}
int icep_learned_set_params(icep_ctx *c, const double *params) {
  return ok(c) && params ? wrap(c, c->e->learned_params(const_cast<double *>(params), false)) : ICEP_ERR_ARG;
}
int icep_learned_forward(icep_ctx *c, const double *eps, const double *r, double eps_ref, double *y) {
  return ok(c) && eps && r && y ? wrap(c, c->e->learned_forward(eps, r, eps_ref, y)) : ICEP_ERR_ARG;
}
int icep_learned_backward(icep_ctx *c, const double *gy, double *grad) {
  return ok(c) && gy && grad ? wrap(c, c->e->learned_backward(gy, grad)) : ICEP_ERR_ARG;
}
int icep_learned_stats(icep_ctx *c, int *fallbacks, int *precond_apps) {
  if (!ok(c)) return ICEP_ERR_ARG;
  if (fallbacks) *fallbacks = c->e->last_fallbacks;
  if (precond_apps) *precond_apps = c->e->last_precond_apps;
  return ICEP_OK;
}

/* ---- batches of independent replicas ------------------------------------ */
}  // extern "C"

struct icep_batch {
  std::vector<icep_ctx *> ctx;
  std::string err;
  // all replicas' steps captured into one CUDA graph (built at the first step
  // that every replica can take as a graph) and its failure, after which the
  // batch steps from the thread pool
  cudaGraphExec_t exec = nullptr;
  bool graph_failed = false;
};

namespace {
// Runs fn(i) for every replica on a pool of host threads; each replica's
// work goes to its own CUDA stream, so the replicas run concurrently on the
// GPU. Returns the first error (its text in b->err).
template <class F>
int batch_run(icep_batch *b, F fn) {
  const int n = (int)b->ctx.size();
  unsigned hw = std::thread::hardware_concurrency();
  const int nt = std::max(1, std::min(n, (int)std::min(hw ? hw : 4u, 32u)));
  std::atomic<int> next{0}, first_err{0}, err_idx{-1};
  auto worker = [&]() {
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= n) break;
      const int st = fn(b->ctx[i]);
      int expected = 0;
      if (st != ICEP_OK && first_err.compare_exchange_strong(expected, st)) err_idx = i;
    }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++) th.emplace_back(worker);
  for (auto &t : th) t.join();
  if (first_err) {
    const int i = err_idx;
    b->err = "replica " + std::to_string(i) + ": " + (i >= 0 ? b->ctx[i]->err : std::string());
  }
  return first_err;
}
}  // namespace

extern "C" {

icep_batch *icep_batch_create(int n, const icep_params *params, const icep_particle *const *particles, int *status) {
  if (n < 1 || !params || !particles) {
    if (status) *status = ICEP_ERR_ARG;
    return nullptr;
  }
  icep_batch *b = new icep_batch();
  for (int i = 0; i < n; i++) {
    int st = ICEP_OK;
    icep_ctx *c = icep_create(&params[i], particles[i], params[i].n_particles, &st);
    if (!c) {
      for (icep_ctx *o : b->ctx) icep_destroy(o);
      delete b;
      if (status) *status = st;
      return nullptr;
    }
    b->ctx.push_back(c);
  }
  if (status) *status = ICEP_OK;
  return b;
}
void icep_batch_destroy(icep_batch *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (icep_ctx *c : b->ctx) icep_destroy(c);
  delete b;
}
int icep_batch_size(const icep_batch *b) { return b ? (int)b->ctx.size() : 0; }
icep_ctx *icep_batch_context(icep_batch *b, int i) {
  return (b && i >= 0 && i < (int)b->ctx.size()) ? b->ctx[i] : nullptr;
}
const char *icep_batch_last_error(const icep_batch *b) { return b ? b->err.c_str() : "null batch"; }
int icep_batch_init_state(icep_batch *b) {
  return b ? batch_run(b, [](icep_ctx *c) { return icep_init_state(c); }) : ICEP_ERR_ARG;
}
namespace {
// One step of every replica as one graph launch: each replica's captured step
// is an independent branch of the batch graph, so the replicas' kernels run
// concurrently with one launch and one host wait per batch step. Returns -1
// when some replica cannot step as a graph now (the caller steps the batch
// from the thread pool instead).
int batch_graph_step(icep_batch *b) {
  if (b->graph_failed) return -1;
  for (icep_ctx *c : b->ctx)
    if (!c->e->whole_step_ok()) return -1;
  cudaStream_t s = b->ctx[0]->e->stream();
  if (!b->exec) {
    cudaGraph_t gr = nullptr;
    int st = cudaGraphCreate(&gr, 0) == cudaSuccess ? ICEP_OK : ICEP_ERR_CUDA;
    for (size_t i = 0; i < b->ctx.size() && st == ICEP_OK; i++) {
      std::vector<cudaGraphNode_t> deps;
      st = b->ctx[i]->e->capture_step(gr, deps);
    }
    if (st == ICEP_OK && cudaGraphInstantiate(&b->exec, gr, 0) != cudaSuccess) st = ICEP_ERR_CUDA;
    if (gr) cudaGraphDestroy(gr);
    if (st != ICEP_OK) {
      cudaGetLastError();
      if (b->exec) cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
      b->graph_failed = true;
      return -1;
    }
  }
  for (icep_ctx *c : b->ctx) c->e->refresh_field();
  // the replicas' streams may still hold earlier work (e.g. their first step)
  for (icep_ctx *c : b->ctx)
    if (cudaStreamSynchronize(c->e->stream()) != cudaSuccess) return ICEP_ERR_CUDA;
  if (cudaGraphLaunch(b->exec, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    b->err = std::string("batch step graph: ") + cudaGetErrorString(cudaGetLastError());
    return ICEP_ERR_CUDA;
  }
  int first = ICEP_OK;
  for (size_t i = 0; i < b->ctx.size(); i++) {
    const int st = wrap(b->ctx[i], b->ctx[i]->e->step_graph_done(true));
    if (st != ICEP_OK && first == ICEP_OK) {
      first = st;
      b->err = "replica " + std::to_string(i) + ": " + b->ctx[i]->err;
    }
  }
  return first;
}
}  // namespace

int icep_batch_step(icep_batch *b, int nsteps) {
  if (!b || nsteps < 0) return ICEP_ERR_ARG;
  for (int k = 0; k < nsteps;) {
    int st = batch_graph_step(b);
    int done = 1;
    if (st < 0) {
      // from the thread pool: one step while a replica takes its first (after
      // which the graph may become possible), else all that remain
      bool first = false;
      for (icep_ctx *c : b->ctx) first = first || c->e->ts == 0;
      done = first ? 1 : nsteps - k;
      st = batch_run(b, [done](icep_ctx *c) {
        const int q = icep_step(c, done);
        return q != ICEP_OK ? q : icep_synchronize(c);
      });
    }
    if (st != ICEP_OK) return st;
    k += done;
  }
  return ICEP_OK;
}

}  // extern "C"
