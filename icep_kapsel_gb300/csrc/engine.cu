// engine.cu -- device state and step orchestration of one ICEP simulation.
//
// The call order of each phase follows the reference function named in its
// comment; kernels live in fft.cu, fields.cu, particles.cu and krylov.cu.
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <random>
#include <utility>
#include <vector>

#include "engine.cuh"
#include "fields.cuh"
#include "krylov.cuh"
#include "kop.cuh"
#include "probe.cuh"
#include "kspace.cuh"
#include "refine.cuh"
#include "solve_graph.cuh"
#include "unet.cuh"
#include <type_traits>

namespace icep {

namespace {

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

template <typename R>
class Engine : public EngineBase {
 public:
  icep_params P;
  Grid g;
  cudaStream_t s = nullptr;
  FFTPlan<R> fft;
  R *f[F_COUNT];
  double *stage = nullptr;  // FP64 staging for get/set of FP32 fields
  // per-field FP64 staging of the batched host I/O (MIXED), allocated on first use
  static constexpr int NSTAGE = 8;
  double *stage_n[NSTAGE] = {nullptr};
  // the FP64 potential last handed to the host (MIXED): a potential passed
  // back unchanged keeps the solver's float-float state
  double *pot_export = nullptr;
  bool pot_export_valid = false;
  int *dflag = nullptr;
  icep_particle *dp = nullptr;
  icep_particle *hp = nullptr;  // pinned
  int np = 0;
  int *dsek = nullptr;
  int npd = 0;
  PartParams pp;
  double *ukdc = nullptr;    // device double[3]
  // E_ext at the current time (times sin(2 pi f t) for an AC field) and the
  // same times NX*NY*NZ (the k = 0 term of Add_constant_field_k)
  double ext_now[3] = {0, 0, 0}, e_ext_nh[3] = {0, 0, 0};
  void refresh_field() override { refresh_ext(); }
  void refresh_ext() {
    const double f = P.ac ? sin(2.0 * M_PI * P.frequency * time) : 1.0;
    const double amp = (double)P.nx * P.ny * P.nz * f;
    for (int d = 0; d < 3; d++) {
      ext_now[d] = P.ac ? P.e_ext[d] * f : P.e_ext[d];
      e_ext_nh[d] = P.e_ext[d] * amp;
    }
  }
  double *partials = nullptr;
  double *scal = nullptr;
  void *shift_tab = nullptr;  // staggered-shift tables referenced by g
  double *kpart = nullptr;    // dot partials of the fused k-space iteration
  double *hkpart = nullptr;   // pinned
  int *kerr = nullptr;        // error word of the fused plane passes (inside kpart)
  double *kfin = nullptr;     // final sums of the three dot passes (inside kpart), then kerr
  double *kst = nullptr;      // device-side iteration state of the fused solver (inside kpart, after kerr)
  int kf_pred = 0;            // iterations of the last fused solve (the first batch of the next)
  unsigned *kcnt = nullptr;   // last-block counters of the dot passes
  int kop_npb = 0;
  KopTiles kop_tiles;        // the autotuner's picks for this mesh
  bool kop_tuned = false;
  // the MIXED inner solve: preconditioned CG (the operator and the spectral
  // preconditioner are symmetric: 17 operator applications per step at
  // 128^3 against BiCGSTAB's 20) or, with ICEP_INNER=bicgstab, BiCGSTAB
  bool inner_cg = true;
  double kop_tune_us[8] = {0};
  // learned preconditioner and its flexible GMRES (solver LEARNED)
  static constexpr int FG_M = 20;  // restart length
  bool learned = false;
  UNet net;
  bool net_trained = false, net_use = true;
  float *fgV[FG_M + 1] = {nullptr}, *fgZ[FG_M] = {nullptr};
  double *kcoef = nullptr, *hcoef = nullptr, *mpart = nullptr;
  enum { KC_H1 = 0, KC_H2 = KVEC_MAX, KC_NRM = 2 * KVEC_MAX, KC_Y = 2 * KVEC_MAX + 1, KC_COUNT = 3 * KVEC_MAX + 1 };
  double *hscal = nullptr;  // pinned
  double *hukdc = nullptr;  // pinned: uk_dc on its way back to the drop-in call
  int *ljwork = nullptr;
  int ljwork_ints = 0;
  int *dpairs_n = nullptr;
  double radius, xi, hxi, nu;
  double valency_e[2], onsager[2];
  bool electrolyte;
  // FP64-accurate shadow of the Poisson problem (MIXED precision only), as
  // float-float vectors (8 bytes per number, the FP64 layout): potential
  // spectrum, right-hand side, residual, operator work fields and the
  // previous potential spectrum.
  enum { D_X = 0, D_B, D_R, D_W3_0, D_W3_1, D_W3_2, D_XP, D_COUNT };
  bool mixed = false;
  bool janus = false;  // Janus permittivity field (particle 0's species has an axis)
  bool have_sc = false;  // charged particles (Conc_k2charge_field with Make_phi_qq_particle)
  bool salt_free = false;  // one ion species (N_spec = 1), the counterions
  // optional per-phase device timing of the step (CUDA events at phase
  // boundaries, accumulated in ms)
  static constexpr int NPH = 10;
  bool phase_on = false;
  cudaEvent_t ph_ev[NPH + 1];
  double ph_ms[NPH] = {0};
  void mark(int k) {
    if (phase_on) cudaEventRecord(ph_ev[k], s);
  }
  FFTPlan<dfl> fftdf;
  RefineTables rtab;
  double *d64[D_COUNT] = {nullptr};
  dfl *df(int i) { return reinterpret_cast<dfl *>(d64[i]); }
  bool x64_valid = false;
  bool xp_valid = false;  // D_XP holds the potential of the previous solve

  // The step's two fixed kernel sequences (before and after the Poisson
  // solve, whose host-side iteration control stays outside) captured once as
  // CUDA graphs and replayed each step: one launch each instead of ~100
  // kernel launches, which is what bounds small replicas. Used when no
  // kernel argument changes between steps (no AC field; no surface charges,
  // whose charge normalisation reads a sum on the host; no phase profiling)
  // from the second step on (the first uses the Euler integrators); disabled
  // by ICEP_GRAPHS=0 and, for the context, by any capture failure (the step
  // then runs eagerly).
  bool use_graphs = false;
  cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
  unsigned long long glaunch[3] = {0, 0, 0}, gbytes[3] = {0, 0, 0};
  template <class Body>
  int run_segment(int k, Body body) {
    if (!use_graphs || ts == 0) return body();
    return run_graph(k, body);
  }
  // body() captured once into graph slot k (0, 1: the step's sequences; 2:
  // one iteration of the fused Poisson solve), then replayed
  template <class Body>
  int run_graph(int k, Body body) {
    if (!gexec[k]) {
      const unsigned long long l0 = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED);
      const unsigned long long b0 = __atomic_load_n(&g_alg_bytes, __ATOMIC_RELAXED);
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        use_graphs = false;
        return body();
      }
      const int st = body();
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamEndCapture(s, &graph);
      const unsigned long long dl = __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED) - l0;
      const unsigned long long db = __atomic_load_n(&g_alg_bytes, __ATOMIC_RELAXED) - b0;
      // nothing captured has run: its counts come with each replay
      __atomic_fetch_sub(&g_kernel_launches, dl, __ATOMIC_RELAXED);
      __atomic_fetch_sub(&g_alg_bytes, db, __ATOMIC_RELAXED);
      if (e == cudaSuccess && st == ICEP_OK) e = cudaGraphInstantiate(&gexec[k], graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (st != ICEP_OK || e != cudaSuccess || !gexec[k]) {
        cudaGetLastError();
        gexec[k] = nullptr;
        use_graphs = false;
        return body();  // the sequence runs eagerly from now on
      }
      glaunch[k] = dl;
      gbytes[k] = db;
    }
    if (cudaGraphLaunch(gexec[k], s) != cudaSuccess) return cuda_status("graph launch");
    __atomic_fetch_add(&g_kernel_launches, glaunch[k], __ATOMIC_RELAXED);
    __atomic_fetch_add(&g_alg_bytes, gbytes[k], __ATOMIC_RELAXED);
    return ICEP_OK;
  }

  // ---- the whole step as one CUDA graph -------------------------------
  // With the MIXED fused solver the solve's loops run on the device
  // (solve_graph.cuh): the step -- the two fixed sequences, the solve with
  // its sweep and iteration loops as conditional WHILE nodes, and a copy of
  // the solve's status to pinned host memory -- is captured once and
  // replayed as one launch, and the host waits once per step. Used where the
  // segment graphs are (use_graphs), for an electrolyte on the fused passes
  // once the potential's float-float history is in place (from the second
  // step after init_state, or after a change of the potential), without the
  // learned preconditioner or a kernel probe; otherwise, and after any
  // capture failure, the step runs as before.
  double *sc = nullptr;         // SC_COUNT doubles, then SCF_COUNT floats (solve_graph.cuh)
  float *scf = nullptr;
  double *hstat = nullptr;      // pinned: sc, then kfin's 7 + KS_COUNT doubles
  cudaGraphExec_t step_exec = nullptr;
  bool step_graph_failed = false;
  // kernel launches and algorithmic bytes of the captured step: outside the
  // loops, per sweep body (outside the inner loop), per inner iteration
  unsigned long long sg_l[3] = {0, 0, 0}, sg_b[3] = {0, 0, 0};
  static unsigned long long launches_now() { return __atomic_load_n(&g_kernel_launches, __ATOMIC_RELAXED); }
  static unsigned long long bytes_now() { return __atomic_load_n(&g_alg_bytes, __ATOMIC_RELAXED); }

  bool whole_step_ok() const override {
    return use_graphs && ts != 0 && mixed && electrolyte && kpart && sc && !learned && x64_valid && xp_valid &&
           g_probe_kind == PROBE_NONE && !step_graph_failed;
  }

  // Appends this context's step to graph gr after the nodes deps (deps
  // receives the step's last nodes). Nothing captured runs: the kernel
  // counters and the host-side counts are restored, and come with each
  // replay (step_graph_done).
  int capture_step(cudaGraph_t gr, std::vector<cudaGraphNode_t> &deps) override {
    if constexpr (!std::is_same<R, float>::value) {
      return ICEP_ERR_UNSUPPORTED;
    } else {
      const long nf = g.nf();
      const double eps2 = DBL_EPSILON * DBL_EPSILON, nreal = (double)g.nreal(), tol = P.potential_tol;
      const int maxit = P.potential_iter;
      const long mv0 = matvecs;
      float *r = f[F_KR], *r0 = f[F_KR0], *p = f[F_KP], *v = f[F_KV];
      const float *prescale = scf + SCF_PRESCALE;
      cudaGraphConditionalHandle hs = 0, hi = 0;
      cudaGraphNode_t ns = nullptr, ni = nullptr;
      cudaGraph_t bs = nullptr, bi = nullptr;
      std::vector<cudaGraphNode_t> sdeps, ideps;
      int st = ICEP_OK;
      cudaError_t e = cudaSuccess;
      unsigned long long cl[3] = {0, 0, 0}, cb[3] = {0, 0, 0};
      // one stream capture appended to `into` after `after` (leaf back in after)
      auto seg = [&](int part, cudaGraph_t into, std::vector<cudaGraphNode_t> &after, auto body) {
        if (e != cudaSuccess || st != ICEP_OK) return;
        const unsigned long long l0 = launches_now(), b0 = bytes_now();
        e = cap_begin(s, into, after);
        if (e != cudaSuccess) return;
        st = body();
        const cudaError_t e2 = cap_end(s, after);
        if (e == cudaSuccess) e = e2;
        cl[part] += launches_now() - l0;
        cb[part] += bytes_now() - b0;
      };
      const bool use[3] = {ext_now[0] != 0.0, ext_now[1] != 0.0, ext_now[2] != 0.0};
      e = cudaGraphConditionalHandleCreate(&hs, gr, 0, cudaGraphCondAssignDefault);
      // the sequence before the solve, the right-hand side, the first true
      // residual and the sweep loop's first decision
      seg(0, gr, deps, [&]() -> int {
        int q = pre_solve();
        if (q) return q;
        rf_extrapolate_shift(nf, df(D_X), df(D_XP), s);
        dfl *w[3] = {df(D_W3_0), df(D_W3_1), df(D_W3_2)};
        rf_eps_face_e(g, w[0], w[1], w[2], (const float *)f[F_EPS], ext_now, use, s);
        FieldBatch<dfl> nz{};
        for (int d = 0; d < 3; d++)
          if (use[d]) nz.p[nz.n++] = w[d];
        if (nz.n) fft_r2c(fftdf, nz, s);
        rf_from_f32(nf, (const float *)f[F_UP0], df(D_R), s);
        fft_r2c(fftdf, batch(df(D_R)), s);
        rf_div_combine(g, rtab, df(D_W3_0), df(D_W3_1), df(D_W3_2), use, df(D_R), df(D_B), RF_RHS, 1.f, true,
                       partials, scal, S_BB, s);
        sum_real<R>(g, f[F_EPS], partials, scal, S_AUX1, s);
        solve_begin(scal, S_BB, S_AUX1, sc, scf, kst, tol, nreal, s);
        kop_eps_faces(g, f[F_EPS], f[F_EF0], f[F_EF1], f[F_EF2], s);
        residual_df(1.f, prescale);
        sweep_cond(hs, scal, S_RR, sc, scf, kst, tol, nreal, 30, false, s);
        return ICEP_OK;
      });
      if (e == cudaSuccess && st == ICEP_OK) e = add_while(gr, deps, hs, &ns, &bs);
      if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hi, bs, 0, cudaGraphCondAssignDefault);
      // a sweep: the FP32 correction problem on the normalised residual
      seg(1, bs, sdeps, [&]() -> int {
        rf_to_f32(nf, df(D_R), r, scf + SCF_INVRN, s);
        cudaMemsetAsync(r, 0, 2 * sizeof(R), s);  // k = 0: the mean
        kdots<R>(g, r, r, r, r, 1, partials, scal, S_RR, s);
        zero(F_KY);
        zero(F_KP);
        if (!inner_cg) {  // BiCGSTAB's shadow residual and v (CG writes q before reading it)
          cudaMemcpyAsync(r0, r, sizeof(R) * nf, cudaMemcpyDeviceToDevice, s);
          zero(F_KV);
        }
        inner_prep(hi, scal, S_RR, sc, kst, eps2, inner_cg, s);
        if (inner_cg) kf_cg_start(maxit);
        return ICEP_OK;
      });
      if (e == cudaSuccess && st == ICEP_OK) e = add_while(bs, sdeps, hi, &ni, &bi);
      sdeps.assign(1, ni);
      seg(2, bi, ideps, [&]() -> int {
        if (inner_cg) {
          kf_cg_iteration(maxit, hi);  // the CG update sets the loop's condition
        } else {
          kf_iteration(1.0, maxit);
          inner_cond(hi, kst, r, r0, v, p, nf, maxit, sc, eps2, s);
        }
        return ICEP_OK;
      });
      // the correction added, the next true residual and decision
      seg(1, bs, sdeps, [&]() -> int {
        kprecond<R>(g, f[F_KY], f[F_KX], kst + KS_IEPS, s);
        rf_add_f32(nf, f[F_KX], df(D_X), reinterpret_cast<const float2 *>(scf + SCF_RN), s);
        residual_df(1.f, prescale);
        sweep_cond(hs, scal, S_RR, sc, scf, kst, tol, nreal, 30, true, s);
        return ICEP_OK;
      });
      deps.assign(1, ns);
      // the potential, the sequence after the solve, the status to the host
      seg(0, gr, deps, [&]() -> int {
        rf_zero_if(nf, df(D_X), sc + SC_ZERO_RHS, s);
        rf_to_f32(nf, df(D_X), (float *)f[F_POT], 1.0, s);
        c2r(f[F_POT]);
        const int q = post_solve();
        if (q) return q;
        cudaMemcpyAsync(hstat, sc, sizeof(double) * SC_COUNT, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hstat + SC_COUNT, kfin, sizeof(double) * (7 + KS_COUNT), cudaMemcpyDeviceToHost, s);
        return ICEP_OK;
      });
      matvecs = mv0;
      __atomic_fetch_sub(&g_kernel_launches, cl[0] + cl[1] + cl[2], __ATOMIC_RELAXED);
      __atomic_fetch_sub(&g_alg_bytes, cb[0] + cb[1] + cb[2], __ATOMIC_RELAXED);
      for (int k = 0; k < 3; k++) {
        sg_l[k] = cl[k];
        sg_b[k] = cb[k];
      }
      if (st != ICEP_OK) return st;
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ICEP_ERR_CUDA, (std::string("capture of the step graph: ") + cudaGetErrorString(e)).c_str());
      }
      return ICEP_OK;
    }
  }
  // After a replay of the captured step (the stream synchronised): the
  // solve's status and counts, and with `advance` the step's time advance.
  int step_graph_done(bool advance) override {
    const double *h = hstat;
    const double *hks = h + SC_COUNT + 7;
    const double sweeps = h[SC_SWEEPS], inner = h[SC_INNER];
    __atomic_fetch_add(&g_kernel_launches,
                       sg_l[0] + (unsigned long long)sweeps * sg_l[1] + (unsigned long long)inner * sg_l[2],
                       __ATOMIC_RELAXED);
    __atomic_fetch_add(&g_alg_bytes,
                       sg_b[0] + (unsigned long long)sweeps * sg_b[1] + (unsigned long long)inner * sg_b[2],
                       __ATOMIC_RELAXED);
    matvecs += (long)(sweeps + 1.0) + (inner_cg ? 1 : 2) * (long)inner;
    last_iters = (int)inner;
    last_error = h[SC_REL];
    last_fallbacks = 0;
    last_precond_apps = 0;
    kf_pred = (int)hks[KS_ITERS];
    pot_export_valid = false;
    graph_steps++;
    if (*reinterpret_cast<const int *>(h + SC_COUNT + 6))
      return fail(ICEP_ERR_TIMEOUT, "plane pass: a bulk copy did not complete within the wait limit");
    if (h[SC_STATUS] != (double)ICEP_OK)
      return fail((int)h[SC_STATUS], "Poisson solve: non-finite right-hand side or residual");
    if (h[SC_GUARD] != 0.0) return fail(ICEP_ERR_NOT_CONVERGED, "Poisson solve: inner loop guard reached");
    if (advance) {
      time += P.dt;
      ts++;
    }
    return cuda_status("step");
  }
  int run_step_graph() {
    if (!step_exec) {
      cudaGraph_t gr = nullptr;
      std::vector<cudaGraphNode_t> deps;
      int st = cudaGraphCreate(&gr, 0) == cudaSuccess ? capture_step(gr, deps) : ICEP_ERR_CUDA;
      if (st == ICEP_OK && cudaGraphInstantiate(&step_exec, gr, 0) != cudaSuccess) st = ICEP_ERR_CUDA;
      if (gr) cudaGraphDestroy(gr);
      if (st != ICEP_OK) {
        cudaGetLastError();
        if (step_exec) cudaGraphExecDestroy(step_exec);
        step_exec = nullptr;
        step_graph_failed = true;  // this context steps as before from now on
        err.clear();
        return time_evolution_hydro();
      }
    }
    if (cudaGraphLaunch(step_exec, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
      return cuda_status("step graph");
    return step_graph_done(false);  // step() advances time and ts
  }

  ~Engine() override {
    if (s) cudaStreamSynchronize(s);
    for (int k = 0; k < 3; k++)
      if (gexec[k]) cudaGraphExecDestroy(gexec[k]);
    if (step_exec) cudaGraphExecDestroy(step_exec);
    cudaFree(sc);
    cudaFreeHost(hstat);
    for (int i = 0; i < F_COUNT; i++) cudaFree(f[i]);
    fft_plan_free(fft);
    for (int i = 0; i < D_COUNT; i++) cudaFree(d64[i]);
    if (mixed) fft_plan_free(fftdf);
    rtab.free_all();
    cudaFree(stage);
    for (int i = 0; i < NSTAGE; i++) cudaFree(stage_n[i]);
    cudaFree(pot_export);
    cudaFree(dflag);
    cudaFree(dp);
    cudaFreeHost(hp);
    cudaFree(dsek);
    cudaFree(ukdc);
    cudaFree(partials);
    cudaFree(scal);
    cudaFree(shift_tab);
    cudaFree(kpart);
    cudaFree(kcnt);
    cudaFreeHost(hkpart);
    if (learned) net.free_all();
    for (int i = 0; i <= FG_M; i++) cudaFree(fgV[i]);
    for (int i = 0; i < FG_M; i++) cudaFree(fgZ[i]);
    cudaFree(kcoef);
    cudaFreeHost(hcoef);
    cudaFree(mpart);
    cudaFreeHost(hscal);
    cudaFreeHost(hukdc);
    cudaFree(ljwork);
    cudaFree(dpairs_n);
    if (phase_on)
      for (int k = 0; k <= NPH; k++) cudaEventDestroy(ph_ev[k]);
    if (s) cudaStreamDestroy(s);
  }

  cudaStream_t stream() const override { return s; }

  int fail(int code, const char *msg) {
    err = msg;
    return code;
  }
  int cuda_status(const char *where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      err = std::string(where) + ": " + cudaGetErrorString(e);
      return ICEP_ERR_CUDA;
    }
    return ICEP_OK;
  }

  int setup(const icep_params &p, const icep_particle *parts, int n) {
    for (int i = 0; i < F_COUNT; i++) f[i] = nullptr;
    P = p;
    if (!pow2(p.nx) || !pow2(p.ny) || !pow2(p.nz) || p.nx < 16 || p.ny < 16 || p.nz < 16 || p.nx > 256 ||
        p.ny > 256 || p.nz > 256)
      return fail(ICEP_ERR_UNSUPPORTED, "mesh sizes must be powers of two in [16, 256]");
    if (n != p.n_particles || n < 0) return fail(ICEP_ERR_ARG, "particle count mismatch");
    if (p.n_species < 1 || p.n_species > ICEP_MAX_SPECIES) return fail(ICEP_ERR_ARG, "n_species out of range");
    if (p.dt <= 0 || p.dx <= 0 || p.rho <= 0 || p.eta <= 0) return fail(ICEP_ERR_ARG, "non-positive dt/dx/rho/eta");
    for (int q = 0; q < n; q++)
      if (parts[q].spec < 0 || parts[q].spec >= p.n_species) return fail(ICEP_ERR_ARG, "particle species out of range");
    // Janus field when particle 0's species has an axis (operate_dielectric.cxx:
    // 276-280); the reference exits when another particle's species has none
    // (operate_dielectric.cxx:195-198)
    for (int q = 0; q < ICEP_MAX_SPECIES; q++)
      if (p.janus_axis[q] < ICEP_JANUS_NONE || p.janus_axis[q] > ICEP_JANUS_Z)
        return fail(ICEP_ERR_ARG, "janus_axis out of range");
    janus = n > 0 && p.janus_axis[parts[0].spec] != ICEP_JANUS_NONE;
    // surface charges: all species charged or none (Init_rho_ion_dielectric,
    // operate_electrolyte.cxx:912-930, exits otherwise)
    have_sc = p.n_species > 0 && p.surface_charge[0] != 0.0;
    for (int q = 0; q < p.n_species; q++)
      if ((p.surface_charge[q] != 0.0) != have_sc)
        return fail(ICEP_ERR_ARG, "surface charges must be non-zero for every species or for none");
    if (have_sc && p.sw_eq != ICEP_ELECTROLYTE) return fail(ICEP_ERR_ARG, "surface charges need the Electrolyte model");
    // salt-free: the counterions of charged particles of one sign, the
    // counterions' valency opposite to it (Init_rho_ion_dielectric's
    // no-charge branch needs two species; Init_rho_ion,
    // operate_electrolyte.cxx:740-787, exits otherwise)
    salt_free = p.sw_eq == ICEP_ELECTROLYTE && p.salt_free != 0;
    if (salt_free) {
      if (!have_sc) return fail(ICEP_ERR_ARG, "salt-free electrolyte needs charged particles");
      for (int q = 0; q < p.n_species; q++)
        if (p.surface_charge[q] * p.surface_charge[0] <= 0.)
          return fail(ICEP_ERR_ARG, "salt-free electrolyte with particles of both signs");
      if (p.valency_counterion * p.surface_charge[0] >= 0.)
        return fail(ICEP_ERR_ARG, "counterion valency must be opposite to the surface charge");
    }
    // INIT_profile Poisson_Boltzmann: with charged particles the reference
    // relaxes the ion densities (Init_rho_ion, operate_electrolyte.cxx:
    // 810-853); built here: the salt solution with more than one particle
    // (Set_steadystate_ion_density); uncharged particles start uniform there
    if (p.poisson_boltzmann && have_sc && (salt_free || n <= 1))
      return fail(ICEP_ERR_UNSUPPORTED,
                  "INIT_profile Poisson_Boltzmann: only the salt solution with more than one charged particle "
                  "(Set_steadystate_ion_density) is built; the salt-free and single-particle relaxations are not");
    if (janus) {
      if (p.per_particle_eps) return fail(ICEP_ERR_ARG, "Janus particles with per-particle permittivity");
      for (int q = 0; q < n; q++)
        if (p.janus_axis[parts[q].spec] == ICEP_JANUS_NONE)
          return fail(ICEP_ERR_ARG, "Janus field: a particle's species has no Janus axis");
    }
    electrolyte = (p.sw_eq == ICEP_ELECTROLYTE);
    if (electrolyte && !p.dielectric)
      return fail(ICEP_ERR_UNSUPPORTED, "Electrolyte requires Dielectric_property ON on this path");
    if (p.sw_eq != ICEP_NAVIER_STOKES && p.sw_eq != ICEP_ELECTROLYTE) return fail(ICEP_ERR_UNSUPPORTED, "SW_EQ");
    g.nx = p.nx; g.ny = p.ny; g.nz = p.nz;
    g.hnz = p.nz / 2 + 1;
    g.nzp = 2 * g.hnz;
    const int N[3] = {p.nx, p.ny, p.nz};
    for (int d = 0; d < 3; d++) {
      g.trn[d] = (N[d] + 2) / 3;
      g.wave[d] = 2.0 * M_PI / (N[d] * p.dx);
      g.wavef[d] = (float)g.wave[d];
    }
    g.dx = p.dx;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      return fail(ICEP_ERR_CUDA, "cudaStreamCreate failed (no GPU?)");
    if (make_shift_tables() != ICEP_OK) return fail(ICEP_ERR_CUDA, "shift tables");
    radius = p.a * p.dx;
    xi = p.a_xi * p.dx;
    hxi = 0.5 * xi;
    nu = p.eta / p.rho;
    valency_e[0] = p.valency_pos * p.elementary_charge;
    valency_e[1] = p.valency_neg * p.elementary_charge;
    onsager[0] = p.onsager_pos;
    onsager[1] = p.onsager_neg;
    if (salt_free) {  // N_spec = 1: the second species is absent (zero)
      valency_e[0] = p.valency_counterion * p.elementary_charge;
      valency_e[1] = 0.0;
      onsager[0] = p.onsager_counterion;
      onsager[1] = 0.0;
    }
    const size_t fb = sizeof(R) * g.nf();
    for (int i = 0; i < F_COUNT; i++) {
      if (cudaMalloc(&f[i], fb) != cudaSuccess) return fail(ICEP_ERR_CUDA, "cudaMalloc of fields failed");
      cudaMemsetAsync(f[i], 0, fb, s);
    }
    if (sizeof(R) != sizeof(double) && cudaMalloc(&stage, sizeof(double) * g.nf()) != cudaSuccess)
      return fail(ICEP_ERR_CUDA, "cudaMalloc of staging failed");
    if (fft_plan_init(fft, g, s) != ICEP_OK) return fail(ICEP_ERR_CUDA, "FFT plan setup failed");
    mixed = (sizeof(R) != sizeof(double));
    if (mixed && electrolyte) {
      for (int i = 0; i < D_COUNT; i++) {
        if (cudaMalloc(&d64[i], sizeof(double) * g.nf()) != cudaSuccess)
          return fail(ICEP_ERR_CUDA, "cudaMalloc of FP64 Poisson fields failed");
        cudaMemsetAsync(d64[i], 0, sizeof(double) * g.nf(), s);
      }
      if (fft_plan_init(fftdf, g, s) != ICEP_OK) return fail(ICEP_ERR_CUDA, "float-float FFT plan setup failed");
      if (rtab.init(g, s) != ICEP_OK) return fail(ICEP_ERR_CUDA, "float-float operator tables");
    }
    // Particle_domain (profile.cxx:25-74)
    std::vector<int> sek;
    const int nh = (int)p.a + (int)p.a_xi + 2;
    const double max_r = radius + hxi + 1.7321 * p.dx;
    for (int i = -nh; i <= nh; i++)
      for (int j = -nh; j <= nh; j++)
        for (int k = -nh; k <= nh; k++) {
          const double d = sqrt((i * p.dx) * (i * p.dx) + (j * p.dx) * (j * p.dx) + (k * p.dx) * (k * p.dx));
          if (d < max_r) {
            sek.push_back(i);
            sek.push_back(j);
            sek.push_back(k);
          }
        }
    npd = (int)(sek.size() / 3);
    if (2 * nh + 1 > p.nx || 2 * nh + 1 > p.ny || 2 * nh + 1 > p.nz)
      return fail(ICEP_ERR_UNSUPPORTED, "particle stencil wider than the box");
    cudaMalloc(&dsek, sizeof(int) * sek.size());
    cudaMemcpyAsync(dsek, sek.data(), sizeof(int) * sek.size(), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);  // sek is a local vector
    np = n;
    cudaMalloc(&dp, sizeof(icep_particle) * (n > 0 ? n : 1));
    cudaMallocHost(&hp, sizeof(icep_particle) * (n > 0 ? n : 1));
    for (int q = 0; q < n; q++) {
      hp[q] = parts[q];
      if (!p.per_particle_eps) hp[q].eps_p = p.eps_particle_top;
    }
    cudaMemcpyAsync(dp, hp, sizeof(icep_particle) * n, cudaMemcpyHostToDevice, s);
    abs_total_qe = 0.0;
    for (int q = 0; q < n; q++) abs_total_qe += fabs(p.surface_charge[hp[q].spec] * p.elementary_charge);
    // particle parameters (Set_global_parameters, input.cxx:286-300, 404-440)
    memset(&pp, 0, sizeof(pp));
    pp.dx = p.dx; pp.radius = radius; pp.xi = xi; pp.hxi = hxi;
    set_band_bounds(pp);
    for (int d = 0; d < 3; d++) {
      pp.L[d] = N[d] * p.dx;
      pp.N[d] = N[d];
    }
    pp.nzp = g.nzp;
    pp.rotation = p.rotation;
    pp.np = n;
    pp.np_domain = npd;
    pp.eps_f = p.eps_fluid;
    pp.dt = p.dt;
    pp.rho = p.rho;
    lj_params_from(p, pp);
    pp.n_species = p.n_species;
    for (int q = 0; q < ICEP_MAX_SPECIES; q++) {
      const double mass = p.mass_ratio[q] * p.rho * 4. / 3. * M_PI * radius * radius * radius;
      pp.imass[q] = (mass > 0) ? 1. / mass : 0.0;
      pp.imoi[q] = (mass > 0) ? 1. / (2. / 5. * mass * radius * radius) : 0.0;
      pp.mass_ratio[q] = p.mass_ratio[q];
      pp.motor[q] = (q < p.n_species && p.janus_propulsion[q] == ICEP_MOTOR) ? 1 : 0;
      for (int d = 0; d < 3; d++) {
        pp.jforce[q][d] = p.janus_force[q][d];
        pp.jtorque[q][d] = p.janus_torque[q][d];
      }
    }
    pp.g = p.g;
    pp.g_direction = p.g_direction;
    for (int q = 0; q < ICEP_MAX_SPECIES; q++) pp.janus_axis[q] = p.janus_axis[q] - 1;  // x, y, z -> 0, 1, 2
    pp.eps_ave = 0.5 * (p.eps_particle_top + p.eps_particle_bottom) * p.dielectric_cst;
    pp.eps_delta = 0.5 * (p.eps_particle_top - p.eps_particle_bottom) * p.dielectric_cst;
    pp.sharp = 1.0 / p.dx;
    for (int q = 0; q < ICEP_MAX_SPECIES; q++) pp.qe[q] = p.surface_charge[q] * p.elementary_charge;
    cudaMalloc(&ukdc, sizeof(double) * 3);
    cudaMemsetAsync(ukdc, 0, sizeof(double) * 3, s);
    refresh_ext();
    cudaMalloc(&partials, sizeof(double) * 2 * DOT_BLOCKS);
    if (mixed && electrolyte && kop_supported(g)) {
      kop_npb = kop_pencil_blocks(g);
      // the dot partials of the three passes, their final sums (3 pairs), then
      // one word for the plane passes' error flag; three pass counters
      // and the device-side iteration state (KS_COUNT doubles)
      const size_t nk = 2 * (2 * (size_t)kop_npb + kop_xr_blocks(g)) + 7 + KS_COUNT;
      if (cudaMalloc(&kpart, sizeof(double) * nk) != cudaSuccess ||
          cudaMallocHost(&hkpart, sizeof(double) * (7 + KS_COUNT)) != cudaSuccess ||
          cudaMalloc(&kcnt, sizeof(unsigned) * 4) != cudaSuccess)
        return fail(ICEP_ERR_CUDA, "allocation of the k-space dot partials failed");
      cudaMemsetAsync(kpart, 0, sizeof(double) * nk, s);
      cudaMemsetAsync(kcnt, 0, sizeof(unsigned) * 4, s);
      kfin = kpart + nk - 7 - KS_COUNT;
      kerr = reinterpret_cast<int *>(kfin + 6);
      kst = kfin + 7;
      // the FP32 transforms' register-resident plane passes report a copy
      // that did not land through the same word
      fft.err = kerr;
      // the device-side control of the solve for step graphs, and its status
      // copy on the host
      if (cudaMalloc(&sc, sizeof(double) * SC_COUNT + sizeof(float) * SCF_COUNT) != cudaSuccess ||
          cudaMallocHost(&hstat, sizeof(double) * (SC_COUNT + 7 + KS_COUNT)) != cudaSuccess)
        return fail(ICEP_ERR_CUDA, "allocation of the solve's control state failed");
      scf = reinterpret_cast<float *>(sc + SC_COUNT);
      cudaMemsetAsync(sc, 0, sizeof(double) * SC_COUNT + sizeof(float) * SCF_COUNT, s);
      // tile choices of the fused passes (cached per mesh); ICEP_AUTOTUNE=0
      // keeps the defaults, ICEP_KOP_TILES="xinv,xfwd,plane" sets them
      const char *at = getenv("ICEP_AUTOTUNE");
      const char *force = getenv("ICEP_KOP_TILES");
      int fi = 0, ff = 0, fp = 0;
      if (force && sscanf(force, "%d,%d,%d", &fi, &ff, &fp) == 3) {
        kop_tiles.xinv_kw = fi;
        kop_tiles.xfwd_kw = ff;
        kop_tiles.plane_smem = fp;
        kop_tuned = true;  // picks set by hand: reported with no timings
      } else if constexpr (std::is_same<R, float>::value) {
        if (!(at && at[0] == '0')) {
          kop_tiles = kop_autotune(fft, f[F_KP], f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], f[F_WV3_3], f[F_EF0], f[F_EF1], f[F_EF2],
                                   f[F_KV], kerr, s, kop_tune_us);
          kop_tuned = true;
        }
      }
    }
    if (p.solver == ICEP_SOLVER_LEARNED) {
      if (!mixed || !electrolyte || !kpart || p.nx != p.ny || p.nx != p.nz || p.nx < 32)
        return fail(ICEP_ERR_UNSUPPORTED,
                    "solver LEARNED needs precision MIXED, Electrolyte, a cubic mesh of 32..128 per axis");
      learned = true;
      if (net.init(p.nx / 2, 0x1ce9u, s) != ICEP_OK) return fail(ICEP_ERR_CUDA, "network setup failed");
      for (int i = 0; i <= FG_M; i++)
        if (cudaMalloc(&fgV[i], sizeof(R) * g.nf()) != cudaSuccess) return fail(ICEP_ERR_CUDA, "GMRES vectors");
      for (int i = 0; i < FG_M; i++)
        if (cudaMalloc(&fgZ[i], sizeof(R) * g.nf()) != cudaSuccess) return fail(ICEP_ERR_CUDA, "GMRES vectors");
      if (cudaMalloc(&kcoef, sizeof(double) * KC_COUNT) != cudaSuccess ||
          cudaMallocHost(&hcoef, sizeof(double) * KC_COUNT) != cudaSuccess ||
          cudaMalloc(&mpart, sizeof(double) * DOT_BLOCKS * KVEC_MAX) != cudaSuccess)
        return fail(ICEP_ERR_CUDA, "GMRES scalars");
    }
    cudaMalloc(&scal, sizeof(double) * S_COUNT);
    cudaMemsetAsync(scal, 0, sizeof(double) * S_COUNT, s);
    cudaMallocHost(&hscal, sizeof(double) * S_COUNT);
    const int ncell = (p.nx / 16) * (p.ny / 16) * (p.nz / 16);
    ljwork_ints = 2 * (ncell + 1) + (n > 0 ? n : 1);
    cudaMalloc(&ljwork, sizeof(int) * ljwork_ints);
    cudaMalloc(&dpairs_n, sizeof(int));
    const char *pe = getenv("ICEP_PHASE_PROFILE");
    if (pe && pe[0] == '1') {
      phase_on = true;
      for (int k = 0; k <= NPH; k++) cudaEventCreate(&ph_ev[k]);
    }
    const char *ie = getenv("ICEP_INNER");
    inner_cg = !(ie && strcmp(ie, "bicgstab") == 0);
    const char *ge = getenv("ICEP_GRAPHS");
    use_graphs = !(ge && ge[0] == '0') && !phase_on && !p.ac && !have_sc;
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("setup");
    return cuda_status("setup");
  }

  // exp(i dx k_d / 2) per wavenumber index, the staggered shifts of the
  // reference's Shift_* tables (fft_wrapper.h:841-900), computed in FP64 on
  // the host; the FP32 copy is the rounded FP64 value
  int make_shift_tables() {
    const int n[3] = {g.nx, g.ny, g.hnz};
    const int tot = n[0] + n[1] + n[2];
    std::vector<double> hd(2 * (size_t)tot);
    std::vector<float> hf(2 * (size_t)tot);
    int off = 0;
    for (int d = 0; d < 3; d++)
      for (int q = 0; q < n[d]; q++, off++) {
        const int kint = (d == 0) ? kx_of(g, q) : (d == 1) ? ky_of(g, q) : q;
        const double a = 0.5 * g.dx * g.wave[d] * kint;
        hd[2 * off] = cos(a);
        hd[2 * off + 1] = sin(a);
        hf[2 * off] = (float)hd[2 * off];
        hf[2 * off + 1] = (float)hd[2 * off + 1];
      }
    const size_t bd = sizeof(double) * hd.size(), bf = sizeof(float) * hf.size();
    if (cudaMalloc(&shift_tab, bd + bf) != cudaSuccess) return ICEP_ERR_CUDA;
    char *base = static_cast<char *>(shift_tab);
    cudaMemcpyAsync(base, hd.data(), bd, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(base + bd, hf.data(), bf, cudaMemcpyHostToDevice, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return ICEP_ERR_CUDA;
    const double2 *dd = reinterpret_cast<const double2 *>(base);
    const float2 *ff = reinterpret_cast<const float2 *>(base + bd);
    g.shd[0] = dd;
    g.shd[1] = dd + n[0];
    g.shd[2] = dd + n[0] + n[1];
    g.shf[0] = ff;
    g.shf[1] = ff + n[0];
    g.shf[2] = ff + n[0] + n[1];
    return ICEP_OK;
  }

  // ---------------------------------------------------------------- helpers
  void zero(int id) { cudaMemsetAsync(f[id], 0, sizeof(R) * g.nf(), s); }
  void copy(int dst, int src) { cudaMemcpyAsync(f[dst], f[src], sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s); }
  void r2c(R *a, R *b = nullptr, R *c = nullptr, R *d = nullptr, R *e = nullptr) {
    fft_r2c(fft, batch(a, b, c, d, e), s);
  }
  void c2r(R *a, R *b = nullptr, R *c = nullptr, R *d = nullptr, R *e = nullptr) {
    fft_c2r(fft, batch(a, b, c, d, e), s);
  }
  R *const *vec(int id0) { return &f[id0]; }

  // Zeta_k2u (operate_omega.h:138-141)
  void zeta_k2u() {
    zeta_k2u_k<R>(g, f[F_ZETA0], f[F_ZETA1], ukdc, f[F_U0], f[F_U1], f[F_U2], s);
    c2r(f[F_U0], f[F_U1], f[F_U2]);
  }
  // Truncate_vector_two_third_rule of zeta then Zeta_k2u, the truncation
  // fused into the k-space pass (fluid_solver.cxx:342-343; sp_3d_ns.cxx:37-38)
  void truncate_zeta_k2u() {
    zeta_k2u_trunc<R>(g, f[F_ZETA0], f[F_ZETA1], ukdc, f[F_U0], f[F_U1], f[F_U2], s);
    c2r(f[F_U0], f[F_U1], f[F_U2]);
  }
  // U2advection_k (operate_omega.cxx:12-98) on real u into adv0/adv1
  void u2advection_k(int a0, int a1) {
    advection_products<R>(g, f[F_U0], f[F_U1], f[F_U2], f[a0], f[a1], s);
    r2c(f[F_U0], f[F_U1], f[F_U2], f[a0], f[a1]);
    advection_combine<R>(g, f[F_U0], f[F_U1], f[F_U2], f[a0], f[a1], s);
  }
  // Solenoidal_u (operate_omega.h:109-116)
  void solenoidal_u(int id0) {
    r2c(f[id0], f[id0 + 1], f[id0 + 2]);
    truncate_solenoidal_uk<R>(g, f[id0], f[id0 + 1], f[id0 + 2], s);
    c2r(f[id0], f[id0 + 1], f[id0 + 2]);
  }
  // NS_solver_slavedEuler (fluid_solver.cxx:340-366)
  void ns_solver_slaved_euler() {
    truncate_zeta_k2u();
    u2advection_k(F_NS0_0, F_NS0_1);
    ns_slaved_update<R>(g, f[F_ZETA0], f[F_ZETA1], f[F_NS0_0], f[F_NS0_1], nu, P.dt, s);
  }
  // Make_phi_particle_sum (make_phi.cxx:229-275)
  void make_phi_particle_sum() {
    zero(F_PHI_SUM);
    scatter_profile<R>(pp, dp, dsek, f[F_PHI_SUM], nullptr, PROF_PHI, s);
    zero(F_PHI);
    phi_clip<R>(g, f[F_PHI_SUM], f[F_PHI], s);
  }
  // Make_u_particle_sum (make_phi.cxx:329-370)
  void make_u_particle_sum() {
    for (int d = 0; d < 3; d++) zero(F_UP0 + d);
    scatter_up<R>(pp, dp, dsek, f[F_PHI_SUM], f[F_UP0], f[F_UP1], f[F_UP2], s);
  }
  // Make_f_particle_dt_sole + Add_f_particle (f_particle.h:37-95) + U2zeta_k
  // (operate_omega.h:212-215): f = up - phi u, then f and u to spectra and
  // one k-space pass (u += P T f, the vorticity and mean flow of the sum).
  // Leaves u as its spectrum, as U2zeta_k does, and f as the spectrum of the
  // non-solenoidal force.
  void f_particle_sole_add_to_zeta() {
    f_nonsole<R>(g, vec(F_F0), vec(F_UP0), f[F_PHI], vec(F_U0), s);
    r2c(f[F_F0], f[F_F1], f[F_F2]);
    r2c(f[F_U0], f[F_U1], f[F_U2]);
    sole_add_zeta<R>(g, vec(F_F0), vec(F_U0), f[F_ZETA0], f[F_ZETA1], ukdc, s);
  }
  // Make_dielectric_field (operate_dielectric.cxx:270-309): phi_sin into
  // phi_id; per-particle permittivity (extension) accumulates into aux_id.
  void make_dielectric_field(int phi_id, int aux_id) {
    zero(phi_id);
    if (janus) {  // Make_janus_permittivity_dielectric (operate_dielectric.cxx:208-267)
      zero(aux_id);
      scatter_profile<R>(pp, dp, dsek, f[phi_id], f[aux_id], PROF_JANUS, s);
      eps_janus<R>(g, f[F_EPS], f[phi_id], f[aux_id], P.eps_fluid, P.dielectric_cst, s);
      return;
    }
    R *aux = nullptr;
    if (P.per_particle_eps) {
      zero(aux_id);
      aux = f[aux_id];
    }
    scatter_profile<R>(pp, dp, dsek, f[phi_id], aux, PROF_PHI_SIN, s);
    eps_from_profile<R>(g, f[F_EPS], f[phi_id], aux, P.eps_fluid, P.eps_particle_top, P.dielectric_cst, s);
  }
  // Conc_k2charge_field_no_surfase_charge (operate_dielectric.cxx:135-160);
  // with surface charges Conc_k2charge_field (operate_electrolyte.cxx:45-74):
  // phi_id becomes the sum of Phi and rho starts from the surface charge of
  // Make_phi_qq_particle (operate_electrolyte.cxx:179-243)
  // (tmp2_id, if given, lets both species' densities go to real space in
  // one batched transform)
  int conc_k2charge(int rho_id, int phi_id, int tmp_id, int tmp2_id = -1) {
    if (have_sc) {
      zero(phi_id);
      zero(rho_id);
      scatter_profile<R>(pp, dp, dsek, f[phi_id], f[rho_id], PROF_QQ, s);
      sum_abs_real<R>(g, f[rho_id], partials, scal, S_AUX1, s);
      int st = read_scal();
      if (st) return st;
      // volume of the surface section normalised to sum_n |e Q_n|
      const double rescale = abs_total_qe / (hscal[S_AUX1] * P.dx * P.dx * P.dx);
      scale_copy<R>(g, f[rho_id], f[rho_id], (R)rescale, s);
    }
    if (tmp2_id >= 0) {
      copy(tmp_id, F_C0);
      copy(tmp2_id, F_C1);
      c2r(f[tmp_id], f[tmp2_id]);
      charge_add2<R>(g, f[rho_id], f[tmp_id], f[tmp2_id], f[phi_id], valency_e[0], valency_e[1], !have_sc, s);
      return ICEP_OK;
    }
    for (int n = 0; n < 2; n++) {
      copy(tmp_id, F_C0 + n);
      c2r(f[tmp_id]);
      charge_add<R>(g, f[rho_id], f[tmp_id], f[phi_id], valency_e[n], n == 0 && !have_sc, s);
    }
    return ICEP_OK;
  }
  double abs_total_qe = 0.0;  // sum over particles of |e Q|
  // Ax (operate_dielectric.cxx:485-522) on padded real fields
  void apply_A(const R *x, R *y) {
    copy_real<R>(g, x, y, s);
    r2c(y);
    grad_k<R>(g, y, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], R(1), true, nullptr, s);
    c2r(f[F_WV3_0], f[F_WV3_1], f[F_WV3_2]);
    eps_face_mul<R>(g, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], f[F_EPS], s);
    r2c(f[F_WV3_0], f[F_WV3_1], f[F_WV3_2]);
    div_k<R>(g, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], y, true, s);
    c2r(y);
    matvecs++;
  }
  // Build_rhs (operate_dielectric.cxx:524-540)
  void build_rhs(int rhs_id, int rho_id) {
    eps_face_E<R>(g, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], f[F_EPS], ext_now[0], ext_now[1], ext_now[2], s);
    FieldBatch<R> nz{};  // zero components of E_ext: cleared (with their padding), not transformed
    for (int d = 0; d < 3; d++) {
      if (ext_now[d] != 0.0) nz.p[nz.n++] = f[F_WV3_0 + d];
      else zero(F_WV3_0 + d);
    }
    if (nz.n) fft_r2c(fft, nz, s);
    div_k<R>(g, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], f[rhs_id], true, s);
    c2r(f[rhs_id]);
    axpby_real<R>(g, f[rho_id], f[rhs_id], R(-1), R(1), s);
  }
  int read_scal() {
    cudaMemcpyAsync(hscal, scal, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("solver sync");
    return ICEP_OK;
  }

  // Spectral preconditioner: y = M^-1 x
  void precond(const R *x, R *y, double eps_ref) {
    copy_real<R>(g, x, y, s);
    r2c(y);
    inv_laplace_k<R>(g, y, eps_ref, s);
    c2r(y);
  }

  /*
   * BiCGSTAB on padded fields F_KB (b) and F_KX (x, guess in / solution out).
   * spectral == false: identity preconditioner, Eigen's stopping rule on the
   * recursively updated residual and its restart rule (the REF solver).
   * spectral == true: right preconditioner M^-1 (constant-eps_ref spectral
   * inverse), b projected onto mean zero (the range of the operator, whose
   * null space is the constants), convergence confirmed on the true residual.
   */
  int bicgstab(double tol, int maxit, bool spectral, double eps_ref, int *iters, double *rel_err) {
    R *b = f[F_KB], *x = f[F_KX], *r = f[F_KR], *r0 = f[F_KR0], *p = f[F_KP], *v = f[F_KV];
    R *sv = f[F_KS], *t = f[F_KT], *y = f[F_KY], *z = f[F_KZ];
    if (spectral) {
      sum_real<R>(g, b, partials, scal, S_AUX0, s);
      sub_mean<R>(g, b, scal, S_AUX0, s);
    }
    apply_A(x, t);
    sub_real<R>(g, b, t, r, s);
    copy_real<R>(g, r, r0, s);
    dots<R>(g, r0, r0, b, b, 2, partials, scal, S_R0R, s);
    int st = read_scal();
    if (st) return st;
    double r0sq = hscal[S_R0R], bsq = hscal[S_R0R + 1];
    if (bsq == 0.0) {
      zero(F_KX);
      *iters = 0;
      *rel_err = 0.0;
      return ICEP_OK;
    }
    zero(F_KV);
    zero(F_KP);
    double rho = 1, alpha = 1, w = 1;
    const double tol2 = tol * tol * bsq, eps2 = DBL_EPSILON * DBL_EPSILON;
    double rr = r0sq, rho_new = r0sq;
    int i = 0, restarts = 0;
    while (i < maxit) {
      if (!(rr > tol2)) {
        if (!spectral) break;
        // confirm on the true residual
        apply_A(x, t);
        sub_real<R>(g, b, t, r, s);
        dots<R>(g, r, r, r, r, 1, partials, scal, S_RR, s);
        if ((st = read_scal())) return st;
        rr = hscal[S_RR];
        if (!(rr > tol2)) break;
        copy_real<R>(g, r, r0, s);
        r0sq = rr;
        rho_new = rr;
        zero(F_KV);
        zero(F_KP);
        rho = 1; alpha = 1; w = 1;
      }
      const double rho_old = rho;
      rho = rho_new;
      if (fabs(rho) < eps2 * r0sq) {
        apply_A(x, t);
        sub_real<R>(g, b, t, r, s);
        copy_real<R>(g, r, r0, s);
        dots<R>(g, r, r, r, r, 1, partials, scal, S_RR, s);
        if ((st = read_scal())) return st;
        rho = r0sq = hscal[S_RR];
        if (restarts++ == 0) i = 0;
      }
      const double beta = (rho / rho_old) * (alpha / w);
      bicg_p<R>(g, p, r, v, beta, w, s);
      const R *yy = p;
      if (spectral) {
        precond(p, y, eps_ref);
        yy = y;
      }
      apply_A(yy, v);
      dots<R>(g, r0, v, r0, v, 1, partials, scal, S_R0V, s);
      bicg_s<R>(g, sv, r, v, rho, scal, s);
      const R *zz = sv;
      if (spectral) {
        precond(sv, z, eps_ref);
        zz = z;
      }
      apply_A(zz, t);
      dots<R>(g, t, t, t, sv, 2, partials, scal, S_TT, s);
      bicg_xr<R>(g, x, r, yy, zz, sv, t, rho, scal, s);
      dots<R>(g, r0, r, r, r, 2, partials, scal, S_R0R, s);
      if ((st = read_scal())) return st;
      alpha = rho / hscal[S_R0V];
      w = (hscal[S_TT] > 0.0) ? hscal[S_TS] / hscal[S_TT] : 0.0;
      rho_new = hscal[S_R0R];
      rr = hscal[S_RR];
      ++i;
      if (!std::isfinite(rr)) break;
    }
    *iters = i;
    *rel_err = sqrt(rr / bsq);
    return ICEP_OK;
  }

  // B = A M^-1 on a k-space vector p into v (the k-space form of A applied
  // to the preconditioned direction; 6 FFTs)
  void apply_B(const R *p, R *v, double eps_ref) {
    kgrad_pre<R>(g, p, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], eps_ref, s);
    c2r(f[F_WV3_0], f[F_WV3_1], f[F_WV3_2]);
    eps_face_mul<R>(g, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], f[F_EPS], s);
    r2c(f[F_WV3_0], f[F_WV3_1], f[F_WV3_2]);
    kdiv_post<R>(g, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], v, s);
    matvecs++;
  }

  /*
   * Right-preconditioned BiCGSTAB held in k-space, from a zero guess: solves
   * A x = b (b: real field in F_KB, its mean removed) and leaves x in F_KX.
   * Same iteration as bicgstab(spectral = true) in exact arithmetic (the
   * vectors are the transforms of the real-space ones and the dot products
   * agree by Parseval), with the preconditioner folded into the operator, so
   * an iteration costs 12 FFTs instead of 20. Stops on the recursive
   * residual; the caller checks the true residual.
   */
  int bicgstab_k(double tol, int maxit, double eps_ref, int *iters, double *rel_err) {
    R *r = f[F_KR], *r0 = f[F_KR0], *p = f[F_KP], *v = f[F_KV];
    R *sv = f[F_KS], *t = f[F_KT], *xt = f[F_KY];
    copy_real<R>(g, f[F_KB], r, s);
    r2c(r);
    cudaMemsetAsync(r, 0, 2 * sizeof(R), s);  // k = 0: the mean
    cudaMemcpyAsync(r0, r, sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
    kdots<R>(g, r, r, r, r, 1, partials, scal, S_RR, s);
    int st = read_scal();
    if (st) return st;
    const double bsq = hscal[S_RR];
    zero(F_KY);
    if (!(bsq > 0.0)) {
      zero(F_KX);
      *iters = 0;
      *rel_err = 0.0;
      return ICEP_OK;
    }
    zero(F_KV);
    zero(F_KP);
    double rho = 1, alpha = 1, w = 1;
    const double tol2 = tol * tol * bsq, eps2 = DBL_EPSILON * DBL_EPSILON;
    double r0sq = bsq, rr = bsq, rho_new = bsq;
    int i = 0;
    while (i < maxit && rr > tol2) {
      const double rho_old = rho;
      rho = rho_new;
      if (fabs(rho) < eps2 * r0sq) {  // restart on the current residual
        cudaMemcpyAsync(r0, r, sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
        rho = r0sq = rr;
        zero(F_KV);
        zero(F_KP);
        alpha = w = 1;
        if (!(rho > 0.0)) break;
        rho_new = rho;
      }
      const double beta = (rho / rho_old) * (alpha / w);
      kbicg_p<R>(g, p, r, v, beta, w, s);
      apply_B(p, v, eps_ref);
      kdots<R>(g, r0, v, r0, v, 1, partials, scal, S_R0V, s);
      kbicg_s<R>(g, sv, r, v, rho, scal, s);
      apply_B(sv, t, eps_ref);
      kdots<R>(g, t, t, t, sv, 2, partials, scal, S_TT, s);
      kbicg_xr<R>(g, xt, r, p, sv, t, rho, scal, s);
      kdots<R>(g, r0, r, r, r, 2, partials, scal, S_R0R, s);
      if ((st = read_scal())) return st;
      alpha = rho / hscal[S_R0V];
      w = (hscal[S_TT] > 0.0) ? hscal[S_TS] / hscal[S_TT] : 0.0;
      rho_new = hscal[S_R0R];
      rr = hscal[S_RR];
      ++i;
      if (!std::isfinite(rr)) break;
    }
    kprecond<R>(g, xt, f[F_KX], eps_ref, s);
    c2r(f[F_KX]);
    *iters = i;
    *rel_err = sqrt(rr / bsq);
    return ICEP_OK;
  }

  /*
   * bicgstab_k with the operator and the vector updates fused into FFT
   * passes (kop.cuh): per iteration 3 passes per operator application plus
   * one update kernel, one host synchronisation. FP32 engine on grids whose
   * x-planes fit in shared memory.
   */
  // One iteration of the fused k-space BiCGSTAB (B x~ = A M^-1 x~ by the
  // fused passes), its scalars in kst; eps_ref is used where kst does not
  // give it.
  void kf_iteration(double eps_ref, int maxit) {
    if constexpr (std::is_same<R, float>::value) {
      float *r = f[F_KR], *r0 = f[F_KR0], *p = f[F_KP], *v = f[F_KV];
      float *sv = f[F_KS], *t = f[F_KT], *xt = f[F_KY];
      float *w0 = f[F_WV3_0], *w1 = f[F_WV3_1], *w2 = f[F_WV3_2], *w3 = f[F_WV3_3];
      const int nb = kop_npb;
      double *P1 = kpart, *P2 = kpart + 2 * nb, *P3 = kpart + 4 * nb;
      double *F1 = kfin, *F2 = kfin + 2, *F3 = kfin + 4;  // final sums; kfin[6] holds the error word
      kop_xinv(fft, KOP_P, p, r, v, 0.0, 0.0, 0.0, nullptr, eps_ref, w0, w1, w2, w3, s, kst, kop_tiles);
      kop_plane(fft, w0, w1, w2, w3, f[F_EF0], f[F_EF1], f[F_EF2], kerr, s, kop_tiles);
      kop_xfwd(fft, w0, w2, w3, v, KOP_P, r0, P1, F1, kcnt, s, kop_tiles);
      kop_xinv(fft, KOP_S, sv, r, v, 0.0, 0.0, 0.0, F1, eps_ref, w0, w1, w2, w3, s, kst, kop_tiles);
      kop_plane(fft, w0, w1, w2, w3, f[F_EF0], f[F_EF1], f[F_EF2], kerr, s, kop_tiles);
      kop_xfwd(fft, w0, w2, w3, t, KOP_S, sv, P2, F2, kcnt + 1, s, kop_tiles);
      kop_xr(g, xt, r, p, sv, t, r0, 0.0, F1, F2, P3, F3, kcnt + 2, s, kst, maxit);
    }
  }
  // One iteration of the fused preconditioned CG (the MIXED inner solve with
  // inner_cg): p~ = r + beta p~ (k_kop_xinv's KOP_PC update) and
  // the gradient of M^-1 p~; the plane pass; q = B p~ into F_KV with the
  // denominator (M^-1 p~, q); the update of x~ and r and the next scalars.
  void kf_cg_iteration(int maxit, cudaGraphConditionalHandle h = 0) {
    if constexpr (std::is_same<R, float>::value) {
      float *r = f[F_KR], *p = f[F_KP], *v = f[F_KV], *xt = f[F_KY];
      float *w0 = f[F_WV3_0], *w1 = f[F_WV3_1], *w2 = f[F_WV3_2], *w3 = f[F_WV3_3];
      const int nb = kop_npb;
      double *P1 = kpart, *P3 = kpart + 4 * nb;
      double *F1 = kfin, *F3 = kfin + 4;
      kop_xinv(fft, KOP_PC, p, r, nullptr, 0.0, 0.0, 0.0, nullptr, 1.0, w0, w1, w2, w3, s, kst, kop_tiles);
      kop_plane(fft, w0, w1, w2, w3, f[F_EF0], f[F_EF1], f[F_EF2], kerr, s, kop_tiles);
      kop_xfwd(fft, w0, w2, w3, v, KOP_CG, p, P1, F1, kcnt, s, kop_tiles, kst);
      kop_cg(g, xt, r, p, v, F1, P3, F3, kcnt + 2, s, kst, maxit, false, h);
    }
  }
  // the CG's starting pass: rho and |r|^2 of the starting residual
  void kf_cg_start(int maxit) {
    if constexpr (std::is_same<R, float>::value) {
      const int nb = kop_npb;
      kop_cg(g, f[F_KY], f[F_KR], f[F_KP], f[F_KV], kfin, kpart + 4 * nb, kfin + 4, kcnt + 2, s, kst, maxit, true);
    }
  }
  int bicgstab_kf(double tol, int maxit, double eps_ref, int *iters, double *rel_err, bool kspace_io = false) {
    if constexpr (!std::is_same<R, float>::value) {
      return bicgstab_k(tol, maxit, eps_ref, iters, rel_err);
    } else {
      float *r = f[F_KR], *r0 = f[F_KR0], *xt = f[F_KY];
      if (!kspace_io) {  // right-hand side from the real field F_KB, else already in F_KR
        copy_real<R>(g, f[F_KB], r, s);
        r2c(r);
      }
      cudaMemsetAsync(r, 0, 2 * sizeof(R), s);  // k = 0: the mean
      cudaMemcpyAsync(r0, r, sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
      kdots<R>(g, r, r, r, r, 1, partials, scal, S_RR, s);
      int st = read_scal();
      if (st) return st;
      const double bsq = hscal[S_RR];
      zero(F_KY);
      if (!(bsq > 0.0)) {
        zero(F_KX);
        *iters = 0;
        *rel_err = 0.0;
        return ICEP_OK;
      }
      zero(F_KV);
      zero(F_KP);
      kop_eps_faces(g, f[F_EPS], f[F_EF0], f[F_EF1], f[F_EF2], s);
      const double tol2 = tol * tol * bsq, eps2 = DBL_EPSILON * DBL_EPSILON;
      double rr = bsq;
      int i = 0;
      // The iteration's scalars live on the device (kst, see kop.cuh): the
      // host enqueues several iterations between synchronisations -- at first
      // as many as the previous solve needed less two (an iteration enqueued
      // past the stop still runs its passes on scratch vectors), then one at
      // a time.
      double *hks = hkpart + 7;
      // BiCGSTAB iteration 0: rho = (r0, r), p = v = 0; CG: p = r (beta =
      // omega = 0), rho from the starting pass
      const bool cg = inner_cg;
      hks[KS_RHO] = bsq;
      hks[KS_BETA] = cg ? 0.0 : 1.0;
      hks[KS_OMEGA] = cg ? 0.0 : 1.0;
      hks[KS_TOL2] = tol2;
      hks[KS_DONE] = 0.0;
      hks[KS_ITERS] = 0.0;
      hks[KS_RR] = bsq;
      hks[KS_RESTART] = cg ? 0.0 : eps2 * bsq;
      hks[KS_IEPS] = 1.0 / eps_ref;
      cudaMemcpyAsync(kst, hks, sizeof(double) * KS_COUNT, cudaMemcpyHostToDevice, s);
      if (cg) kf_cg_start(maxit);
      // one iteration: every argument is a fixed pointer or constant (the
      // scalars, 1/eps_ref and the stop flag live in kst), so it is captured
      // once as a CUDA graph and replayed (not while a probe times launches)
      auto iteration = [&]() -> int {
        if (cg) kf_cg_iteration(maxit);
        else kf_iteration(eps_ref, maxit);
        return ICEP_OK;
      };
      const bool graph_iter = use_graphs && g_probe_kind == PROBE_NONE;
      while (i < maxit && rr > tol2) {
        int chunk = (i == 0 && kf_pred > 2) ? kf_pred - 2 : 1;
        if (chunk > maxit - i) chunk = maxit - i;
        for (int q = 0; q < chunk; q++) {
          if ((st = graph_iter ? run_graph(2, iteration) : iteration())) return st;
        }
        cudaMemcpyAsync(hkpart, kfin, sizeof(double) * (7 + KS_COUNT), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("fused k-space iteration");
        if (*reinterpret_cast<const int *>(hkpart + 6))
          return fail(ICEP_ERR_TIMEOUT, "plane pass: a bulk copy did not complete within the wait limit");
        const int now = (int)hks[KS_ITERS];
        matvecs += (cg ? 1 : 2) * (now - i);
        i = now;
        rr = hks[KS_RR];
        if (!std::isfinite(rr)) break;
        if (hks[KS_DONE] == 2.0) {  // restart on the current residual
          cudaMemcpyAsync(r0, r, sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
          zero(F_KV);
          zero(F_KP);
          if (!(rr > 0.0)) break;
          hks[KS_RHO] = rr;
          hks[KS_BETA] = 1.0;
          hks[KS_OMEGA] = 1.0;
          hks[KS_RESTART] = eps2 * rr;
          hks[KS_DONE] = 0.0;
          cudaMemcpyAsync(kst, hks, sizeof(double) * KS_COUNT, cudaMemcpyHostToDevice, s);
          continue;
        }
        if (hks[KS_DONE] != 0.0) break;
      }
      kf_pred = i;
      kprecond<R>(g, xt, f[F_KX], eps_ref, s);
      if (!kspace_io) c2r(f[F_KX]);
      *iters = i;
      *rel_err = sqrt(rr / bsq);
      return ICEP_OK;
    }
  }

  // ---- learned preconditioner ------------------------------------------
  // P(v) = M^-1 (v + c), c = rms(v) prolong(net(eps, v)) the network's
  // correction of the residual (for the unit-norm k-space vector v); in the
  // x~ form of the fused operator: x~ = v^ + c^, B x~ = A P(v).
  void learned_precond(const float *vhat, float *xt, double eref) {
    if constexpr (std::is_same<R, float>::value) {
      if (!(net_trained && net_use)) {
        cudaMemcpyAsync(xt, vhat, sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
        return;
      }
      const double rms = 1.0 / sqrt((double)g.nreal());  // v has unit norm
      cudaMemcpyAsync(f[F_KZ], vhat, sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
      c2r(f[F_KZ]);
      unet_input(g, f[F_EPS], f[F_KZ], eref, rms, net.x, s);
      net.forward(s);
      zero(F_WV1);
      unet_prolong_add(g, net.y, rms, f[F_WV1], s);
      r2c(f[F_WV1]);
      kadd(g, vhat, f[F_WV1], xt, s);
    }
  }
  // out = B x~ through the fused passes (no vector update, no dots)
  void apply_Bk(float *xt, float *out) {
    if constexpr (std::is_same<R, float>::value) {
      kop_xinv(fft, KOP_NONE, xt, nullptr, nullptr, 0, 0, 0, nullptr, mean_eps_cached, f[F_WV3_0], f[F_WV3_1],
               f[F_WV3_2], f[F_WV3_3], s, nullptr, kop_tiles);
      kop_plane(fft, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], f[F_WV3_3], f[F_EF0], f[F_EF1], f[F_EF2], kerr, s,
                kop_tiles);
      kop_xfwd(fft, f[F_WV3_0], f[F_WV3_2], f[F_WV3_3], out, KOP_NONE, nullptr, nullptr, nullptr, nullptr, s,
               kop_tiles);
      matvecs++;
    }
  }
  double mean_eps_cached = 1.0;
  // |w|^2 (Parseval) into kcoef[slot] on the device
  void knorm2(const float *w, int slot) {
    KVecs one{};
    one.p[0] = w;
    kmdot(g, one, 1, w, mpart, s);
    kmdot_final(mpart, 1, kcoef + slot, s);
  }

  /*
   * Flexible GMRES(FG_M) in k-space on B x~ = b^ (b: F_KB, real, mean
   * removed), right-preconditioned by learned_precond; classical Gram-Schmidt
   * applied twice, FP64 dot products, one host synchronisation per
   * iteration. Converges on the GMRES residual estimate; returns false in
   * *ok when the residual stagnates across a restart or maxit is reached
   * (the caller falls back to the plain solver). Leaves x = M^-1 x~ in F_KX.
   */
  int fgmres(double tol, int maxit, double eref, int *iters, double *rel_err, bool *ok) {
    if constexpr (!std::is_same<R, float>::value) {
      return ICEP_ERR_UNSUPPORTED;
    } else {
      float *bhat = f[F_KR0], *r = f[F_KR], *xt = f[F_KY];
      copy_real<R>(g, f[F_KB], r, s);
      r2c(r);
      cudaMemsetAsync(r, 0, 2 * sizeof(R), s);
      cudaMemcpyAsync(bhat, r, sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
      kop_eps_faces(g, f[F_EPS], f[F_EF0], f[F_EF1], f[F_EF2], s);
      mean_eps_cached = eref;
      knorm2(r, KC_NRM);
      cudaMemcpyAsync(hcoef, kcoef, sizeof(double) * KC_COUNT, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("fgmres");
      double beta = sqrt(hcoef[KC_NRM]);
      const double b0 = beta;
      zero(F_KY);
      *ok = true;
      if (!(beta > 0.0)) {
        zero(F_KX);
        *iters = 0;
        *rel_err = 0.0;
        return ICEP_OK;
      }
      double H[FG_M + 1][FG_M], cs[FG_M], sn[FG_M], gv[FG_M + 1], y[FG_M];
      int total = 0, apps = 0;
      bool conv = false;
      double resid = beta, prev_beta = beta;
      while (total < maxit && !conv) {
        kscale_by_norm(g, r, fgV[0], kcoef + KC_NRM, s);
        for (int i = 0; i <= FG_M; i++) gv[i] = 0.0;
        gv[0] = beta;
        int j = 0;
        for (; j < FG_M && total < maxit; j++) {
          learned_precond(fgV[j], fgZ[j], eref);
          apps++;
          apply_Bk(fgZ[j], fgV[j + 1]);
          KVecs Vs{};
          for (int i = 0; i <= j; i++) Vs.p[i] = fgV[i];
          kmdot(g, Vs, j + 1, fgV[j + 1], mpart, s);
          kmdot_final(mpart, j + 1, kcoef + KC_H1, s);
          kmaxpy(g, fgV[j + 1], Vs, j + 1, kcoef + KC_H1, -1.0, s);
          kmdot(g, Vs, j + 1, fgV[j + 1], mpart, s);
          kmdot_final(mpart, j + 1, kcoef + KC_H2, s);
          kmaxpy(g, fgV[j + 1], Vs, j + 1, kcoef + KC_H2, -1.0, s);
          knorm2(fgV[j + 1], KC_NRM);
          kscale_by_norm(g, fgV[j + 1], fgV[j + 1], kcoef + KC_NRM, s);
          cudaMemcpyAsync(hcoef, kcoef, sizeof(double) * KC_Y, cudaMemcpyDeviceToHost, s);
          if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("fgmres iteration");
          for (int i = 0; i <= j; i++) H[i][j] = hcoef[KC_H1 + i] + hcoef[KC_H2 + i];
          H[j + 1][j] = sqrt(std::max(hcoef[KC_NRM], 0.0));
          for (int i = 0; i < j; i++) {  // previous rotations
            const double a = H[i][j], b = H[i + 1][j];
            H[i][j] = cs[i] * a + sn[i] * b;
            H[i + 1][j] = -sn[i] * a + cs[i] * b;
          }
          const double a = H[j][j], b = H[j + 1][j];
          const double rr = std::hypot(a, b);
          cs[j] = (rr > 0) ? a / rr : 1.0;
          sn[j] = (rr > 0) ? b / rr : 0.0;
          H[j][j] = rr;
          H[j + 1][j] = 0.0;
          gv[j + 1] = -sn[j] * gv[j];
          gv[j] = cs[j] * gv[j];
          total++;
          resid = fabs(gv[j + 1]);
          if (!std::isfinite(resid)) {
            *ok = false;
            break;
          }
          if (resid <= tol * b0) {
            j++;
            conv = true;
            break;
          }
        }
        if (!*ok) break;
        for (int i = j - 1; i >= 0; i--) {  // H y = g
          double t = gv[i];
          for (int k2 = i + 1; k2 < j; k2++) t -= H[i][k2] * y[k2];
          y[i] = (H[i][i] != 0.0) ? t / H[i][i] : 0.0;
        }
        for (int i = 0; i < j; i++) hcoef[KC_Y + i] = y[i];
        cudaMemcpyAsync(kcoef + KC_Y, hcoef + KC_Y, sizeof(double) * j, cudaMemcpyHostToDevice, s);
        KVecs Zs{};
        for (int i = 0; i < j; i++) Zs.p[i] = fgZ[i];
        kmaxpy(g, xt, Zs, j, kcoef + KC_Y, 1.0, s);
        if (conv) break;
        // restart from the true k-space residual
        apply_Bk(xt, fgV[0]);
        ksub(g, bhat, fgV[0], r, s);
        knorm2(r, KC_NRM);
        cudaMemcpyAsync(hcoef, kcoef, sizeof(double) * KC_Y, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("fgmres restart");
        beta = sqrt(std::max(hcoef[KC_NRM], 0.0));
        resid = beta;
        if (!(beta < 0.9 * prev_beta)) {  // stagnation across a restart
          *ok = false;
          break;
        }
        prev_beta = beta;
        if (beta <= tol * b0) conv = true;
      }
      if (!conv) *ok = false;
      {
        int herr[2] = {0, 0};
        cudaMemcpyAsync(&herr[0], kerr, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (net.err) cudaMemcpyAsync(&herr[1], net.err, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("fgmres");
        if (herr[0]) return fail(ICEP_ERR_TIMEOUT, "plane pass: a bulk copy did not complete within the wait limit");
        if (herr[1])
          return fail(ICEP_ERR_TIMEOUT, "network convolution: tensor-core completion did not arrive within the wait limit");
      }
      kprecond<R>(g, xt, f[F_KX], eref, s);
      c2r(f[F_KX]);
      *iters = total;
      *rel_err = resid / b0;
      last_precond_apps += apps;
      return ICEP_OK;
    }
  }

  // random sphere centres in [0, L)^3 with periodic separation >= dmin
  bool random_positions(std::mt19937_64 &rng, double dmin) {
    const double L[3] = {g.nx * P.dx, g.ny * P.dx, g.nz * P.dx};
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::vector<double> c;
    for (int q = 0; q < np; q++) {
      bool placed = false;
      for (int tries = 0; tries < 20000 && !placed; tries++) {
        double x[3];
        for (int d = 0; d < 3; d++) x[d] = u(rng) * L[d];
        placed = true;
        for (int o = 0; o < q && placed; o++) {
          double r2 = 0;
          for (int d = 0; d < 3; d++) {
            double dd = fabs(x[d] - c[3 * o + d]);
            dd = std::min(dd, L[d] - dd);
            r2 += dd * dd;
          }
          placed = r2 >= dmin * dmin;
        }
        if (placed) {
          for (int d = 0; d < 3; d++) {
            c.push_back(x[d]);
            hp[q].x[d] = hp[q].x_nopbc[d] = x[d];
          }
        }
      }
      if (!placed) return false;
    }
    return true;
  }

  // z = P(r) for the unit-norm real residual r (F_KR) into F_KZ: the spectral
  // inverse of r plus, with use_net, the network's correction of r
  void learned_precond_real(double eref, bool use_net) {
    const double rms = 1.0 / sqrt((double)g.nreal());
    copy_real<R>(g, f[F_KR], f[F_KZ], s);
    if (use_net) {
      if constexpr (std::is_same<R, float>::value) {
        unet_input(g, f[F_EPS], f[F_KR], eref, rms, net.x, s);
        net.forward(s);
        unet_prolong_add(g, net.y, rms, f[F_KZ], s);
      }
    }
    precond(f[F_KZ], f[F_KZ], eref);
  }

  // one training step on the unit-norm residual in F_KR (real):
  // loss = |r - A P(r)|^2; dL/dc = -2 M^-1 A (r - A P(r)) for the correction c.
  // Leaves the normalised next residual (r - A P(r))/|.| in F_KR.
  int train_step(double eref, float lr, double *loss) {
    if constexpr (std::is_same<R, float>::value) {
      const double rms = 1.0 / sqrt((double)g.nreal());
      learned_precond_real(eref, true);
      apply_A(f[F_KZ], f[F_KT]);
      sub_real<R>(g, f[F_KR], f[F_KT], f[F_KS], s);
      dots<R>(g, f[F_KS], f[F_KS], f[F_KS], f[F_KS], 1, partials, scal, S_AUX0, s);
      apply_A(f[F_KS], f[F_KT]);
      precond(f[F_KT], f[F_KT], eref);
      unet_prolong_adjoint(g, f[F_KT], -2.0 * rms, net.gy, s);
      net.backward(s);
      net.adam_step(lr, s);
      int st = read_scal();
      if (st) return st;
      *loss = hscal[S_AUX0];
      const double nrm = sqrt(*loss);
      scale_copy<R>(g, f[F_KS], f[F_KR], (R)(nrm > 0 ? 1.0 / nrm : 0.0), s);
    }
    return ICEP_OK;
  }

  // Mean one-step loss |r - A P(r)|^2 of the spectral-only and the learned
  // preconditioner on the same residuals: the context's right-hand side
  // (normalised) and the next chain-1 residuals of the spectral iteration.
  int learned_eval(int chain, double *loss_spectral, double *loss_learned) override {
    if (!learned) return unsupported_learned();
    if (chain < 1) return fail(ICEP_ERR_ARG, "learned_eval chain");
    const double eref = mean_eps();
    build_rhs(F_KB, F_RHO);
    dots<R>(g, f[F_KB], f[F_KB], f[F_KB], f[F_KB], 1, partials, scal, S_AUX0, s);
    sum_real<R>(g, f[F_KB], partials, scal, S_AUX1, s);
    int st = read_scal();
    if (st) return st;
    sub_mean<R>(g, f[F_KB], scal, S_AUX1, s);
    dots<R>(g, f[F_KB], f[F_KB], f[F_KB], f[F_KB], 1, partials, scal, S_AUX0, s);
    if ((st = read_scal())) return st;
    scale_copy<R>(g, f[F_KB], f[F_KB], (R)(1.0 / sqrt(hscal[S_AUX0])), s);
    double ls = 0, ll = 0;
    for (int k = 0; k < chain; k++) {
      double l[2];
      // without a trained network both are the spectral preconditioner
      for (int use = net_trained ? 1 : 0; use >= 0; use--) {
        copy_real<R>(g, f[F_KB], f[F_KR], s);
        learned_precond_real(eref, use == 1 && net_trained);
        apply_A(f[F_KZ], f[F_KT]);
        sub_real<R>(g, f[F_KR], f[F_KT], f[F_KS], s);
        dots<R>(g, f[F_KS], f[F_KS], f[F_KS], f[F_KS], 1, partials, scal, S_AUX0, s);
        if ((st = read_scal())) return st;
        l[use] = hscal[S_AUX0];
      }
      if (!net_trained) l[1] = l[0];
      ls += l[0];
      ll += l[1];
      // next residual of the spectral chain (F_KS holds it after use = 0)
      scale_copy<R>(g, f[F_KS], f[F_KB], (R)(1.0 / sqrt(l[0])), s);
    }
    *loss_spectral = ls / chain;
    *loss_learned = ll / chain;
    return ICEP_OK;
  }

  int learned_train(int configs, int steps, unsigned seed, double lr, double *loss_first, double *loss_last) override {
    if (!learned) return unsupported_learned();
    if (configs < 1 || steps < 1 || !(lr > 0)) return fail(ICEP_ERR_ARG, "learned_train arguments");
    std::vector<icep_particle> keep(np > 0 ? np : 1);
    std::vector<float> snap(net.nparams);  // the parameters before this training
    cudaMemcpyAsync(snap.data(), net.params, sizeof(float) * net.nparams, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hp, dp, sizeof(icep_particle) * np, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("learned_train");
    memcpy(keep.data(), hp, sizeof(icep_particle) * np);
    const double e_keep[3] = {P.e_ext[0], P.e_ext[1], P.e_ext[2]};
    const int ac_keep = P.ac;
    P.ac = 0;  // training fields are DC fields of random direction
    double emag = sqrt(e_keep[0] * e_keep[0] + e_keep[1] * e_keep[1] + e_keep[2] * e_keep[2]);
    if (!(emag > 0)) emag = 0.1;
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    int st = ICEP_OK;
    double loss = 0.0;
    for (int c = 0; c < configs && st == ICEP_OK; c++) {
      if (!random_positions(rng, 2.0 * P.a * P.dx + P.dx)) {
        st = fail(ICEP_ERR_ARG, "cannot place the training particles");
        break;
      }
      // eps_p uniform in [1, 10]; with per-particle permittivities a
      // configuration also draws how many particles it has (np/4 .. np): the
      // others take the fluid's permittivity and are absent from eps
      const int active = P.per_particle_eps ? np / 4 + (int)(u(rng) * (np - np / 4 + 1)) : np;
      for (int q = 0; q < np; q++)
        hp[q].eps_p = !P.per_particle_eps ? P.eps_particle_top : (q < active ? 1.0 + 9.0 * u(rng) : P.eps_fluid);
      cudaMemcpyAsync(dp, hp, sizeof(icep_particle) * np, cudaMemcpyHostToDevice, s);
      double e[3] = {nd(rng), nd(rng), nd(rng)};
      const double en = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
      for (int d = 0; d < 3; d++) P.e_ext[d] = emag * e[d] / en;
      refresh_ext();
      make_dielectric_field(F_WORK, F_WV1);
      const double eref = mean_eps();
      zero(F_KT);
      build_rhs(F_KR, F_KT);  // b = D^-(eps_face E), no free charge
      dots<R>(g, f[F_KR], f[F_KR], f[F_KR], f[F_KR], 1, partials, scal, S_AUX0, s);
      if ((st = read_scal())) break;
      scale_copy<R>(g, f[F_KR], f[F_KR], (R)(1.0 / sqrt(hscal[S_AUX0])), s);
      for (int k = 0; k < steps && st == ICEP_OK; k++) {
        st = train_step(eref, (float)lr, &loss);
        if (c == 0 && k == 0 && loss_first) *loss_first = loss;
      }
    }
    if (loss_last) *loss_last = loss;
    // the context's own state back
    for (int d = 0; d < 3; d++) P.e_ext[d] = e_keep[d];
    P.ac = ac_keep;
    refresh_ext();
    memcpy(hp, keep.data(), sizeof(icep_particle) * np);
    cudaMemcpyAsync(dp, hp, sizeof(icep_particle) * np, cudaMemcpyHostToDevice, s);
    make_dielectric_field(F_WORK, F_WV1);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("learned_train");
    if (st != ICEP_OK) return st;
    // keep the trained parameters only if they lower the one-step loss on
    // the context's own residuals (configurations it was not trained on),
    // over the chain of four residuals that learned_eval(4) reports;
    // otherwise restore the parameters it had before
    net_trained = true;
    double ls = 0.0, ll = 0.0;
    if ((st = learned_eval(4, &ls, &ll))) return st;
    if (!(ll < ls)) {
      // not better than the spectral preconditioner alone: the network is
      // not applied (as before any training), its earlier parameters back
      cudaMemcpyAsync(net.params, snap.data(), sizeof(float) * net.nparams, cudaMemcpyHostToDevice, s);
      net.pack(s);
      net_trained = false;
      kept_training = false;
    } else {
      kept_training = true;
    }
    return cuda_status("learned_train");
  }
  bool kept_training = false;
  int learned_enable(int on) override {
    if (!learned) return unsupported_learned();
    net_use = on != 0;
    if (on) net_trained = true;  // parameters set by the caller count as trained
    return ICEP_OK;
  }
  long learned_nparams() override { return learned ? net.nparams : 0; }
  int learned_params(double *buf, bool get) override {
    if (!learned) return unsupported_learned();
    std::vector<float> h(net.nparams);
    if (get) {
      cudaMemcpyAsync(h.data(), net.params, sizeof(float) * net.nparams, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("learned_params");
      for (long q = 0; q < net.nparams; q++) buf[q] = h[q];
    } else {
      for (long q = 0; q < net.nparams; q++) h[q] = (float)buf[q];
      cudaMemcpyAsync(net.params, h.data(), sizeof(float) * net.nparams, cudaMemcpyHostToDevice, s);
      net.pack(s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("learned_params");
    }
    return ICEP_OK;
  }
  // network on host fine fields (padded layout): y (coarse n^3)
  int learned_forward(const double *eps, const double *r, double eps_ref, double *y) override {
    if (!learned) return unsupported_learned();
    int st;
    if ((st = set_field(F_WORK, eps)) || (st = set_field(F_KR, r))) return st;
    if constexpr (std::is_same<R, float>::value) {
      dots<R>(g, f[F_KR], f[F_KR], f[F_KR], f[F_KR], 1, partials, scal, S_AUX0, s);
      if ((st = read_scal())) return st;
      const double rms = sqrt(hscal[S_AUX0] / (double)g.nreal());
      unet_input(g, f[F_WORK], f[F_KR], eps_ref, rms, net.x, s);
      net.forward(s);
      const long nc = (long)net.n * net.n * net.n;
      std::vector<float> h(nc);
      cudaMemcpyAsync(h.data(), net.y, sizeof(float) * nc, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("learned_forward");
      for (long q = 0; q < nc; q++) y[q] = h[q];
    }
    return ICEP_OK;
  }
  int learned_backward(const double *gy, double *grad) override {
    if (!learned) return unsupported_learned();
    const long nc = (long)net.n * net.n * net.n;
    std::vector<float> h(std::max(nc, net.nparams));
    for (long q = 0; q < nc; q++) h[q] = (float)gy[q];
    cudaMemcpyAsync(net.gy, h.data(), sizeof(float) * nc, cudaMemcpyHostToDevice, s);
    net.backward(s);
    cudaMemcpyAsync(h.data(), net.grads, sizeof(float) * net.nparams, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("learned_backward");
    for (long q = 0; q < net.nparams; q++) grad[q] = h[q];
    return ICEP_OK;
  }

  double mean_eps() {
    sum_real<R>(g, f[F_EPS], partials, scal, S_AUX1, s);
    if (read_scal()) return 1.0;
    return hscal[S_AUX1] / (double)g.nreal();
  }

  // r^ = b^ - A x^ in float-float and |r^|^2 / N into hscal[S_RR] after the
  // next read_scal (A: Ax, operate_dielectric.cxx:485-522, on the FP32
  // permittivity; 6 float-float FFTs)
  void residual_df(float prescale, const float *prescale_dev = nullptr) {
    const bool all[3] = {true, true, true};
    dfl *w0 = df(D_W3_0), *w1 = df(D_W3_1), *w2 = df(D_W3_2);
    rf_grad(g, rtab, df(D_X), w0, w1, w2, s);
    // inverse transforms, times the face permittivity, forward transforms
    fft_c2r_eps_r2c(fftdf, batch(w0, w1, w2), (const float *)f[F_EPS], s);
    rf_div_combine(g, rtab, w0, w1, w2, all, df(D_B), df(D_R), RF_RESIDUAL, prescale, false, partials, scal, S_RR,
                   s, prescale_dev);
    matvecs++;
  }

  /*
   * MIXED precision Charge_field2potential_dielectric: iterative refinement
   * held in k-space. The accurate system is A x = b with A the reference
   * operator on the permittivity eps and b = D^-.(eps_face E) - rho with its
   * mean (the k = 0 mode) removed, both evaluated in float-float arithmetic
   * (48-bit significands) on the FP32 pipes: GB300's FP64 rate is 1/64 of its
   * FP32 rate. The potential's half spectrum x^ is float-float state kept
   * between steps. Each outer step forms the true residual r^ = b^ - A x^
   * (its norm by Parseval) and, while |r| > tol |b|, solves A d = r/|r| in
   * FP32 with the k-space BiCGSTAB to a tolerance that leaves a factor-2
   * margin (the FP32 recursive residual tracks the true one closely at these
   * levels; a cycle that still ends above tol is followed by another), then
   * x^ += |r| d^. The real FP32 potential is one FP32 inverse transform of x^
   * at the end.
   */
  int solve_potential_mixed(int rho_id, int pot_id) {
    const Grid &G = g;
    const long nf = G.nf();
    pot_export_valid = false;
    if (!x64_valid) {
      rf_from_f32(nf, (const float *)f[pot_id], df(D_X), s);
      fft_r2c(fftdf, batch(df(D_X)), s);
      x64_valid = true;
      xp_valid = false;
    }
    // initial guess: the potential extrapolated linearly in time from the
    // last two solves (the reference starts from the last potential; both
    // are converged to the same true-residual tolerance)
    if (xp_valid) {
      rf_extrapolate_shift(nf, df(D_X), df(D_XP), s);
    } else {
      cudaMemcpyAsync(d64[D_XP], d64[D_X], sizeof(double) * nf, cudaMemcpyDeviceToDevice, s);
    }
    xp_valid = true;
    // b^: components of E_ext that are zero give zero fields and are skipped
    const bool use[3] = {ext_now[0] != 0.0, ext_now[1] != 0.0, ext_now[2] != 0.0};
    {
      dfl *w[3] = {df(D_W3_0), df(D_W3_1), df(D_W3_2)};
      rf_eps_face_e(G, w[0], w[1], w[2], (const float *)f[F_EPS], ext_now, use, s);
      FieldBatch<dfl> nz{};
      for (int d = 0; d < 3; d++)
        if (use[d]) nz.p[nz.n++] = w[d];
      if (nz.n) fft_r2c(fftdf, nz, s);
    }
    rf_from_f32(nf, (const float *)f[rho_id], df(D_R), s);
    fft_r2c(fftdf, batch(df(D_R)), s);
    rf_div_combine(G, rtab, df(D_W3_0), df(D_W3_1), df(D_W3_2), use, df(D_R), df(D_B), RF_RHS, 1.f, true, partials,
                   scal, S_BB, s);
    int st = read_scal();
    if (st) return st;
    const double bb = hscal[S_BB];
    if (!std::isfinite(bb)) return fail(ICEP_ERR_NOT_CONVERGED, "Poisson solve: non-finite right-hand side");
    const double eref = mean_eps();
    int total_inner = 0;
    double rel = 0.0;
    last_fallbacks = 0;
    last_precond_apps = 0;
    if (bb > 0.0) {
      const double tol2 = P.potential_tol * P.potential_tol * bb;
      // residual norms are summed in FP32 after scaling by a power of two
      // that brings sum_k |b^_k|^2 to order 1
      // (the exponent kept well inside FP32's range: a right-hand side at
      // round-off level, e.g. uniform fields, must not overflow the scale)
      int pe = -ilogb(sqrt((double)G.nreal() * bb));
      pe = pe < -100 ? -100 : pe > 100 ? 100 : pe;
      const float prescale = (float)ldexp(1.0, pe);
      for (int outer = 0; outer < 30; outer++) {
        residual_df(prescale);
        if ((st = read_scal())) return st;
        const double rr = hscal[S_RR];
        rel = sqrt(rr / bb);
        if (!std::isfinite(rr)) return fail(ICEP_ERR_NOT_CONVERGED, "Poisson solve: non-finite residual");
        if (!(rr > tol2)) break;
        // FP32 correction solve on the normalised residual
        const double rn = sqrt(rr / (double)G.nreal());
        rf_to_f32(nf, df(D_R), (float *)f[F_KR], 1.0 / rn, s);
        double inner_tol = INNER_MARGIN * P.potential_tol * sqrt(bb / rr);
        if (inner_tol < 2e-5) inner_tol = 2e-5;
        if (inner_tol > 0.5) inner_tol = 0.5;
        int it = 0;
        double er = 0.0;
        if (kpart && !learned) {
          if ((st = bicgstab_kf(inner_tol, P.potential_iter, eref, &it, &er, true))) return st;
        } else {  // solvers with a real-space interface
          copy(F_KB, F_KR);
          c2r(f[F_KB]);
          zero(F_KX);
          if (learned) {
            bool ok = true;
            if ((st = fgmres(inner_tol, P.potential_iter, eref, &it, &er, &ok))) return st;
            if (!ok) {  // stagnation: the plain solver from a zero guess
              last_fallbacks++;
              int it2 = 0;
              if ((st = bicgstab_kf(inner_tol, P.potential_iter, eref, &it2, &er))) return st;
              it += it2;
            }
          } else if ((st = bicgstab_k(inner_tol, P.potential_iter, eref, &it, &er))) {
            return st;
          }
          r2c(f[F_KX]);
        }
        total_inner += it;
        rf_add_f32(nf, (const float *)f[F_KX], df(D_X), rn, s);
      }
    } else {
      // b = 0 (e.g. an AC field at a zero crossing with no free charge):
      // x = 0, as the reference's BiCGSTAB returns for a zero right-hand side
      cudaMemsetAsync(d64[D_X], 0, sizeof(double) * nf, s);
    }
    rf_to_f32(nf, df(D_X), (float *)f[pot_id], 1.0, s);
    c2r(f[pot_id]);
    last_iters = total_inner;
    last_error = rel;
    return ICEP_OK;
  }

  // Charge_field2potential_dielectric_LO (operate_dielectric.cxx:542-572)
  int solve_potential(int rho_id, int pot_id, int rhs_id) {
    if (mixed) return solve_potential_mixed(rho_id, pot_id);
    build_rhs(rhs_id, rho_id);
    copy_real<R>(g, f[rhs_id], f[F_KB], s);
    copy_real<R>(g, f[pot_id], f[F_KX], s);
    int it = 0;
    double er = 0.0;
    int st;
    const bool spectral = (P.solver == ICEP_SOLVER_SPECTRAL);
    const double eref = spectral ? mean_eps() : 1.0;
    if ((st = bicgstab(P.potential_tol, P.potential_iter, spectral, eref, &it, &er))) return st;
    if (it == P.potential_iter) {  // retry from a zero guess (operate_dielectric.cxx:563-570)
      zero(F_KX);
      copy_real<R>(g, f[rhs_id], f[F_KB], s);
      if ((st = bicgstab(P.potential_tol, P.potential_iter, spectral, eref, &it, &er))) return st;
    }
    last_iters = it;
    last_error = er;
    if (!std::isfinite(er)) return fail(ICEP_ERR_NOT_CONVERGED, "Poisson solve: non-finite residual");
    copy_real<R>(g, f[F_KX], f[pot_id], s);
    return ICEP_OK;
  }

  // Make_Maxwell_force_x_on_fluid (operate_dielectric.cxx:611-764)
  int maxwell_force(int rho_id) {
    make_dielectric_field(F_F0, F_WORK);
    int st = conc_k2charge(rho_id, F_F0, F_F1, F_F2);
    if (st) return st;
    st = solve_potential(rho_id, F_POT, F_F2);
    if (st) return st;
    maxwell_stress(rho_id);
    return ICEP_OK;
  }
  // the part of Make_Maxwell_force_x_on_fluid after the Poisson solve
  // (operate_dielectric.cxx:651-763)
  // (the force on the fluid into F_F0..2 and a copy into F_GE0..2)
  void maxwell_stress(int rho_id) {
    maxwell_face_force(rho_id);
    interp_normal_to<R>(g, vec(F_WV3_0), vec(F_F0), vec(F_GE0), nullptr, R(0), s);
  }
  // the face force into F_WV3_0..2 (operate_dielectric.cxx:651-755)
  void maxwell_face_force(int rho_id) {
    // the staggered gradients of eps (F_GE0..2) and of the potential
    // (F_F0..2), both spectra from one batched transform (F_KT is free after
    // the solve)
    copy(F_WV1, F_EPS);
    copy(F_KT, F_POT);
    r2c(f[F_WV1], f[F_KT]);
    grad_k<R>(g, f[F_WV1], f[F_GE0], f[F_GE1], f[F_GE2], R(1), true, nullptr, s);
    grad_k<R>(g, f[F_KT], f[F_F0], f[F_F1], f[F_F2], R(1), true, nullptr, s);
    c2r(f[F_GE0], f[F_GE1], f[F_GE2]);
    c2r(f[F_F0], f[F_F1], f[F_F2]);
    maxwell_e2<R>(g, f[F_F0], f[F_F1], f[F_F2], f[F_WV1], ext_now[0], ext_now[1], ext_now[2], P.external_field, s);
    maxwell_face<R>(g, vec(F_F0), vec(F_WV3_0), f[rho_id], f[F_WV1], vec(F_GE0), ext_now[0], ext_now[1], ext_now[2],
                    P.external_field, s);
  }

  // NSsolute_solver_Euler (fluid_solver.cxx:318-338), Dielectric branch of
  // Rhs_NS_Nernst_Planck (:246-292) and Rhs_NS_solute (:184-230)
  void nssolute_solver_euler() {
    // staggered grad of the potential minus E_ext, interpolated to nodes
    copy(F_WV1, F_POT);
    r2c(f[F_WV1]);
    grad_k<R>(g, f[F_WV1], f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], R(1), true, P.external_field ? e_ext_nh : nullptr, s);
    c2r(f[F_WV3_0], f[F_WV3_1], f[F_WV3_2]);
    interp_normal<R>(g, vec(F_F0), vec(F_WV3_0), s);
    truncate_zeta_k2u();
    for (int d = 0; d < 3; d++) zero(F_SN0 + d);
    scatter_normal<R>(pp, dp, dsek, f[F_SN0], f[F_SN1], f[F_SN2], s);
    for (int n = 0; n < (salt_free ? 1 : 2); n++) {  // F_CRHS1 stays zero without a second species
      // truncation, Diffusion_flux_single's grad(kBT L c) and the copy of c
      // whose real values the electric and advective fluxes take, one pass
      grad_trunc_copy<R>(g, f[F_C0 + n], f[F_UP0], f[F_UP1], f[F_UP2], f[F_CRHS0 + n], (R)(P.kbt * onsager[n]), s);
      c2r(f[F_UP0], f[F_UP1], f[F_UP2], f[F_CRHS0 + n]);
      np_flux<R>(g, vec(F_UP0), f[F_CRHS0 + n], vec(F_F0), onsager[n] * valency_e[n], vec(F_SN0), vec(F_U0), s);
      r2c(f[F_UP0], f[F_UP1], f[F_UP2]);
      div_k<R>(g, f[F_UP0], f[F_UP1], f[F_UP2], f[F_CRHS0 + n], false, s);
    }
    u2advection_k(F_NS1_0, F_NS1_1);
    euler_update<R>(g, f[F_ZETA0], f[F_ZETA1], f[F_NS1_0], f[F_NS1_1], f[F_C0], f[F_C1], f[F_CRHS0], f[F_CRHS1],
                    nu, P.dt, s);
  }

  int lj_into_fr() {
    if (!pp.lj_on) return ICEP_OK;
    return lj_force(pp, dp, ljwork, ljwork_ints, nullptr, 0, nullptr, s);
  }

  // Time_evolution_hydro (sp_3d_ns.cxx:24-186): the sequence before the
  // Poisson solve
  int pre_solve() {
    mark(0);
    if (!electrolyte) ns_solver_slaved_euler();
    else nssolute_solver_euler();
    for (int d = 0; d < 3; d++)  // FIX_CELL: time-dependent mean pressure gradient (sp_3d_ns.cxx:30-36)
      if ((P.fix_cell >> d) & 1) cudaMemsetAsync(ukdc + d, 0, sizeof(double), s);
    mark(1);
    truncate_zeta_k2u();
    if (!P.fixed_particle) md_position(pp, dp, ts != 0, s);
    make_phi_particle_sum();
    mark(2);
    if (electrolyte) {
      for (int d = 0; d < 3; d++) {
        zero(F_UP0 + d);
        zero(F_F0 + d);
      }
      f_hydro<R>(pp, dp, dsek, f[F_PHI_SUM], f[F_U0], f[F_U1], f[F_U2], true, s);
      make_dielectric_field(F_F0, F_WORK);
      return conc_k2charge(F_UP0, F_F0, F_F1, F_F2);
    }
    return ICEP_OK;
  }
  // the sequence after it
  int post_solve() {
    if (electrolyte) {
      maxwell_face_force(F_UP0);
      mark(5);
      // the force to nodes, kept in F_GE0..2 and added as u += dt/rho f
      interp_normal_to<R>(g, vec(F_WV3_0), nullptr, vec(F_GE0), vec(F_U0), (R)(P.dt / P.rho), s);
      solenoidal_u(F_U0);
    } else {
      mark(5);
    }
    mark(6);
    f_hydro<R>(pp, dp, dsek, f[F_PHI_SUM], f[F_U0], f[F_U1], f[F_U2], false, s);
    if (!P.fixed_particle) {
      const int s2 = lj_into_fr();
      if (s2) return fail(s2, "LJ cell list");
      md_velocity(pp, dp, ts != 0, s);
    }
    mark(7);
    make_u_particle_sum();
    mark(8);
    f_particle_sole_add_to_zeta();
    return ICEP_OK;
  }

  int time_evolution_hydro() {
    if (whole_step_ok()) return run_step_graph();
    int st;
    st = run_segment(0, [&]() -> int { return pre_solve(); });
    if (st) return st;
    if (electrolyte) {
      mark(3);
      if ((st = solve_potential(F_UP0, F_POT, F_F2))) return st;
      mark(4);
    } else {
      mark(3);
      mark(4);
    }
    st = run_segment(1, [&]() -> int { return post_solve(); });
    if (st) return st;
    mark(9);
    mark(10);
    if (phase_on) {
      cudaEventSynchronize(ph_ev[10]);
      for (int k = 0; k < NPH; k++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ph_ev[k], ph_ev[k + 1]);
        ph_ms[k] += t;
      }
    }
    return cuda_status("step");
  }

  // Count_single_solute (solute_rhs.cxx:130-148) of a real field:
  // sum (1 - phi) c DX^3, as sum c - sum phi c
  double count_solute(const R *conc_x) {
    sum_real<R>(g, conc_x, partials, scal, S_AUX0, s);
    dots<R>(g, f[F_PHI], conc_x, nullptr, nullptr, 1, partials, scal, S_AUX1, s);
    read_scal();
    return (hscal[S_AUX0] - hscal[S_AUX1]) * P.dx * P.dx * P.dx;
  }
  // The Dielectric branch of Calc_free_energy_PB (operate_electrolyte.cxx:
  // 302-421): `charge` is the array the reference accumulates into (its
  // up[1]) and is modified as there; F_PHI holds the particle profile.
  double free_energy_pb(R *charge) {
    R *c0 = f[F_GE1], *c1 = f[F_GE2], *ideal = f[F_WV1], *es = f[F_WORK];
    copy(F_GE1, F_C0);
    copy(F_GE2, F_C1);
    c2r(c0, c1);
    pb_energy_terms<R>(g, c0, c1, f[F_PHI], charge, f[F_POT], valency_e[0], valency_e[1], ext_now, P.dx,
                       P.external_field, ideal, es, s);
    sum_real<R>(g, ideal, partials, scal, S_AUX0, s);
    sum_real<R>(g, es, partials, scal, S_AUX1, s);
    read_scal();
    const double dx3 = P.dx * P.dx * P.dx;
    return hscal[S_AUX0] * P.kbt * dx3 + hscal[S_AUX1] * dx3;
  }
  // Set_steadystate_ion_density (operate_electrolyte.cxx:424-457): the salt
  // densities relaxed by Ion_diffusion_solver_Euler (fluid_solver.cxx:
  // 293-316) -- the Nernst-Planck right-hand side with the fluid at rest and
  // the potential as it is (zero before the first solve: the external field
  // alone drives the ions), an Euler step of the densities on the 2/3 modes
  // and Rescale_solute (solute_rhs.cxx:99-128) back to the initial totals --
  // until the free energy changes by less than TOL = 1e-4
  // (operate_electrolyte.h:22), at most 9999 steps. The free energy's charge
  // array starts as the particle velocity field's y component (the
  // reference's up[1]) and, inside the loop, as the last species' real
  // density before its rescale (Rescale_solute's working array is up[1]).
  int steadystate_ions(const double *total) {
    R *charge = f[F_GE0], *tmp = f[F_U0];
    copy(F_GE0, F_UP1);
    double f_prev = free_energy_pb(charge);
    for (int d = 0; d < 2; d++) {  // zero vorticity and its right-hand side for the density-only Euler step
      zero(F_NS0_0 + d);
      zero(F_NS1_0 + d);
    }
    pb_iterations = 0;
    for (int m = 1; m < 10000; m++) {
      copy(F_WV1, F_POT);
      r2c(f[F_WV1]);
      grad_k<R>(g, f[F_WV1], f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], R(1), true, P.external_field ? e_ext_nh : nullptr, s);
      c2r(f[F_WV3_0], f[F_WV3_1], f[F_WV3_2]);
      interp_normal<R>(g, vec(F_F0), vec(F_WV3_0), s);
      for (int d = 0; d < 3; d++) zero(F_SN0 + d);
      scatter_normal<R>(pp, dp, dsek, f[F_SN0], f[F_SN1], f[F_SN2], s);
      for (int n = 0; n < 2; n++) {
        grad_trunc_copy<R>(g, f[F_C0 + n], f[F_UP0], f[F_UP1], f[F_UP2], f[F_CRHS0 + n], (R)(P.kbt * onsager[n]), s);
        c2r(f[F_UP0], f[F_UP1], f[F_UP2], f[F_CRHS0 + n]);
        np_flux<R>(g, vec(F_UP0), f[F_CRHS0 + n], vec(F_F0), onsager[n] * valency_e[n], vec(F_SN0), nullptr, s);
        r2c(f[F_UP0], f[F_UP1], f[F_UP2]);
        div_k<R>(g, f[F_UP0], f[F_UP1], f[F_UP2], f[F_CRHS0 + n], false, s);
      }
      euler_update<R>(g, f[F_NS0_0], f[F_NS0_1], f[F_NS1_0], f[F_NS1_1], f[F_C0], f[F_C1], f[F_CRHS0], f[F_CRHS1],
                      nu, P.dt, s);
      for (int n = 0; n < 2; n++) {  // Rescale_solute; tmp ends as species 1 before its rescale
        cudaMemcpyAsync(tmp, f[F_C0 + n], sizeof(R) * g.nf(), cudaMemcpyDeviceToDevice, s);
        c2r(tmp);
        const double factor = total[n] / count_solute(tmp);
        scale_copy<R>(g, f[F_C0 + n], f[F_C0 + n], (R)factor, s);
      }
      copy(F_GE0, F_U0);
      const double f_now = free_energy_pb(charge);
      pb_iterations = m;
      if (!std::isfinite(f_now)) return fail(ICEP_ERR_NOT_CONVERGED, "Poisson-Boltzmann initialisation: non-finite free energy");
      if (fabs(f_now - f_prev) < 1e-4) break;
      f_prev = f_now;
    }
    for (int d = 0; d < 3; d++) zero(F_U0 + d);  // the reference leaves the velocity field reset
    return cuda_status("steadystate_ions");
  }
  int pb_iterations = 0;

  // Init_rho_ion_dielectric without surface charge (operate_electrolyte.cxx:864-979)
  int init_ions() {
    zero(F_PHI);
    scatter_profile<R>(pp, dp, dsek, f[F_PHI], nullptr, PROF_PHI, s);
    const double z0 = P.valency_pos, z1 = P.valency_neg;
    double rho_inf = P.kbt * P.dielectric_cst * P.eps_fluid /
                     ((P.elementary_charge * P.debye_length * radius) * (P.elementary_charge * P.debye_length * radius));
    double cp = rho_inf / (z0 * (z0 - z1)), cm = -rho_inf / (z1 * (z0 - z1));
    if (have_sc) {
      // Init_rho_ion -> Set_uniform_ion_charge_density_salt (operate_electrolyte.cxx:
      // 738-862, 559-620): the counterions of the surface charges spread over
      // the fluid volume sum(1 - Phi), plus kBT Dc eps_f / (e lambda_D)^2
      // of salt (this branch has no radius factor)
      double pos = 0.0, neg = 0.0;
      for (int sp = 0; sp < P.n_species; sp++) {
        int cnt = 0;
        for (int q = 0; q < np; q++) cnt += (hp[q].spec == sp);
        const double qs = P.surface_charge[sp], num = (double)cnt;
        if (qs < 0.) pos += fabs(qs * num / z0);
        else if (qs > 0.) neg += fabs(qs * num / z1);
      }
      sum_real<R>(g, f[F_PHI], partials, scal, S_AUX1, s);
      read_scal();
      const double volume_phi = (double)g.nreal() - hscal[S_AUX1];
      const double dx3 = P.dx * P.dx * P.dx;
      rho_inf = P.kbt * P.dielectric_cst / ((P.elementary_charge * P.debye_length) * (P.elementary_charge * P.debye_length));
      rho_inf *= P.eps_fluid;
      cp = pos / (volume_phi * dx3) + rho_inf / (z0 * (z0 - z1));
      cm = neg / (volume_phi * dx3) + -rho_inf / (z1 * (z0 - z1));
      if (salt_free) {
        // Set_uniform_ion_charge_density_nosalt (operate_electrolyte.cxx:459-493):
        // Counterion_number = -sum_i Surface_charge_i N_i / Valency_counterion
        // over the fluid volume, the same density everywhere
        double surface_ion_number = 0.;
        for (int sp = 0; sp < P.n_species; sp++) {
          int cnt = 0;
          for (int q = 0; q < np; q++) cnt += (hp[q].spec == sp);
          surface_ion_number -= P.surface_charge[sp] * cnt;
        }
        const double counterion_number = surface_ion_number / P.valency_counterion;
        cp = counterion_number / (volume_phi * dx3);
        cm = 0.0;
      }
    }
    double total[2];
    for (int n = 0; n < 2; n++) {
      zero(F_C0 + n);
      fill_real<R>(g, f[F_C0 + n], (R)(n ? cm : cp), s);
      total[n] = count_solute(f[F_C0 + n]);
      r2c(f[F_C0 + n]);
    }
    // INIT_profile Poisson_Boltzmann with charged particles in the salt
    // solution and more than one particle (Init_rho_ion,
    // operate_electrolyte.cxx:834-853)
    if (P.poisson_boltzmann && have_sc && !salt_free && np > 1) return steadystate_ions(total);
    return ICEP_OK;
  }

  // ------------------------------------------------------------ interface
  int init_state() override {
    // x_nopbc = x (Init_Particle, init_particle.cxx:389)
    cudaMemcpyAsync(hp, dp, sizeof(icep_particle) * np, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int q = 0; q < np; q++)
      for (int d = 0; d < 3; d++) hp[q].x_nopbc[d] = hp[q].x[d];
    cudaMemcpyAsync(dp, hp, sizeof(icep_particle) * np, cudaMemcpyHostToDevice, s);
    // Init_zeta_k (init_fluid.cxx:10-26): fluid at rest
    zero(F_ZETA0);
    zero(F_ZETA1);
    cudaMemsetAsync(ukdc, 0, sizeof(double) * 3, s);
    // sp_3d_ns.cxx:431-446
    make_phi_particle_sum();
    make_u_particle_sum();
    zeta_k2u();
    f_particle_sole_add_to_zeta();
    cudaMemsetAsync(ukdc, 0, sizeof(double) * 3, s);
    if (electrolyte) {
      time = 0.0;  // Init_potential_dielectric runs at jikan.time = 0
      refresh_ext();
      for (int d = 0; d < 3; d++) zero(F_GE0 + d);
      int st0 = init_ions();
      if (st0) return st0;
      // Init_potential_dielectric (operate_dielectric.cxx:574-609)
      make_dielectric_field(F_GE2, F_WORK);
      int st = conc_k2charge(F_GE1, F_GE2, F_GE0);
      if (st) return st;
      st = solve_potential(F_GE1, F_POT, F_GE2);
      if (st) return st;
    }
    ts = 0;
    time = 0.0;
    return cuda_status("init_state");
  }

  int step(int n) override {
    for (int k = 0; k < n; k++) {
      refresh_ext();  // E_ext sin(Angular_Frequency jikan.time) of an AC field
      int st = time_evolution_hydro();
      if (st) return st;
      time += P.dt;
      ts++;
    }
    return ICEP_OK;
  }

  int get_field(int id, double *host) override {
    if (id < 0 || id >= F_COUNT) return fail(ICEP_ERR_ARG, "field id");
    if (id == F_POT && mixed && x64_valid) {  // the potential is float-float state (its half spectrum)
      if (export_potential(stage)) return ICEP_ERR_CUDA;
      cudaMemcpyAsync(host, stage, sizeof(double) * g.nf(), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("get_field");
      return ICEP_OK;
    }
    if (sizeof(R) == sizeof(double)) {
      cudaMemcpyAsync(host, f[id], sizeof(double) * g.nf(), cudaMemcpyDeviceToHost, s);
    } else {
      convert_f2d(g.nf(), (const float *)f[id], stage, s);
      cudaMemcpyAsync(host, stage, sizeof(double) * g.nf(), cudaMemcpyDeviceToHost, s);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("get_field");
    return ICEP_OK;
  }
  // the FP64 potential from the float-float spectrum into out (device), kept
  // as pot_export for the unchanged-potential test of set_field
  int export_potential(double *out) {
    if (!pot_export && cudaMalloc(&pot_export, sizeof(double) * g.nf()) != cudaSuccess) return 1;
    cudaMemcpyAsync(d64[D_R], d64[D_X], sizeof(double) * g.nf(), cudaMemcpyDeviceToDevice, s);
    fft_c2r(fftdf, batch(df(D_R)), s);
    rf_to_f64(g.nf(), df(D_R), out, s);
    cudaMemcpyAsync(pot_export, out, sizeof(double) * g.nf(), cudaMemcpyDeviceToDevice, s);
    pot_export_valid = true;
    return 0;
  }
  // a potential uploaded into dev (FP64) that equals the last exported one
  // leaves the state as it is; else it replaces the potential and the
  // solver's float-float state. Synchronises the stream.
  int import_potential(const double *dev) {
    bool same = false;
    if (mixed && x64_valid && pot_export_valid) {
      if (!dflag && cudaMalloc(&dflag, sizeof(int)) != cudaSuccess) return cuda_status("set_field");
      rf_differs(g.nf(), dev, pot_export, dflag, s);
      int h = 1;
      cudaMemcpyAsync(&h, dflag, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("set_field");
      same = (h == 0);
    }
    if (same) return ICEP_OK;
    x64_valid = xp_valid = pot_export_valid = false;
    if (sizeof(R) == sizeof(double)) cudaMemcpyAsync(f[F_POT], dev, sizeof(double) * g.nf(), cudaMemcpyDefault, s);
    else link_d2f(g.nf(), dev, (float *)f[F_POT], s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("set_field");
    return ICEP_OK;
  }
  double *stage_buf(int k) {
    if (k >= NSTAGE) return nullptr;
    if (!stage_n[k] && cudaMalloc(&stage_n[k], sizeof(double) * g.nf()) != cudaSuccess) return nullptr;
    return stage_n[k];
  }
  // Host arrays pinned through icep_pin_host are read and written by the
  // conversion kernels themselves over the CPU-GPU link (no staging copy);
  // others go through device staging buffers and the copy engines.
  int set_fields(const int *ids, const double *const *host, int n) override {
    const int st = put_fields(ids, host, n);
    if (st) return st;
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("set_fields");
    return ICEP_OK;
  }
  int get_fields(const int *ids, double *const *host, int n) override {
    const int st = fetch_fields(ids, host, n);
    if (st) return st;
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("get_fields");
    return ICEP_OK;
  }
  int time_evolution_host(const int *ids, double *const *host, int n, double *uk_dc, icep_particle *parts,
                          int nsteps) override {
    if (!hukdc && cudaMallocHost(&hukdc, sizeof(double) * 3) != cudaSuccess)
      return fail(ICEP_ERR_CUDA, "pinned uk_dc buffer");
    int st;
    // a pageable source is consumed before cudaMemcpyAsync returns
    cudaMemcpyAsync(ukdc, uk_dc, sizeof(double) * 3, cudaMemcpyHostToDevice, s);
    if ((st = put_particles(parts)) || (st = put_fields(ids, host, n)) || (st = step(nsteps)) ||
        (st = fetch_fields(ids, host, n)))
      return st;
    cudaMemcpyAsync(hukdc, ukdc, sizeof(double) * 3, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(hp, dp, sizeof(icep_particle) * np, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("time_evolution");
    for (int d = 0; d < 3; d++) uk_dc[d] = hukdc[d];
    memcpy(parts, hp, sizeof(icep_particle) * np);
    return ICEP_OK;
  }
  // set_fields / get_fields without the final synchronisation (the copies
  // and conversion kernels queued on the context's stream)
  int put_fields(const int *ids, const double *const *host, int n) {
    const long nf = g.nf();
    const double *pot_src = nullptr;
    for (int k = 0; k < n; k++) {
      if (ids[k] < 0 || ids[k] >= F_COUNT) return fail(ICEP_ERR_ARG, "field id");
      if (sizeof(R) == sizeof(double) && !(ids[k] == F_POT && mixed)) {
        cudaMemcpyAsync(f[ids[k]], host[k], sizeof(double) * nf, cudaMemcpyHostToDevice, s);
        continue;
      }
      const double *src = static_cast<const double *>(host_mapped(host[k], sizeof(double) * nf));
      if (!src) {
        double *st = stage_buf(k);
        if (!st) return fail(ICEP_ERR_CUDA, "staging buffers");
        cudaMemcpyAsync(st, host[k], sizeof(double) * nf, cudaMemcpyHostToDevice, s);
        src = st;
      }
      if (ids[k] == F_POT && mixed) pot_src = src;
      else link_d2f(nf, src, (float *)f[ids[k]], s);
    }
    if (pot_src) return import_potential(pot_src);  // synchronises
    return ICEP_OK;
  }
  int fetch_fields(const int *ids, double *const *host, int n) {
    const long nf = g.nf();
    for (int k = 0; k < n; k++) {
      if (ids[k] < 0 || ids[k] >= F_COUNT) return fail(ICEP_ERR_ARG, "field id");
      if (sizeof(R) == sizeof(double)) {
        cudaMemcpyAsync(host[k], f[ids[k]], sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
        continue;
      }
      double *dst = static_cast<double *>(host_mapped(host[k], sizeof(double) * nf));
      if (ids[k] == F_POT && mixed && x64_valid) {
        double *st = stage_buf(k);
        if (!st) return fail(ICEP_ERR_CUDA, "staging buffers");
        if (export_potential(st)) return fail(ICEP_ERR_CUDA, "potential export");
        if (dst) link_copy(nf, st, dst, s);
        else cudaMemcpyAsync(host[k], st, sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
      } else if (dst) {
        link_f2d(nf, (const float *)f[ids[k]], dst, s);
      } else {
        double *st = stage_buf(k);
        if (!st) return fail(ICEP_ERR_CUDA, "staging buffers");
        convert_f2d(nf, (const float *)f[ids[k]], st, s);
        cudaMemcpyAsync(host[k], st, sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
      }
    }
    return ICEP_OK;
  }
  // The fields of Output_dielectric_charge_field_data (output.cxx:262-320)
  // with vel, phi and charge printed, into host FP64 arrays (NULL skips):
  // u = Zeta_k2u(zeta, uk_dc); phi = the sum of Phi and the surface charge
  // of Make_phi_qq_particle (operate_electrolyte.cxx:179-243) times 4 pi a^2;
  // the solute charge e sum_n z_n c_n (1 - phi); the potential; eps. The
  // step state is not touched: the work goes to the Krylov work vectors.
  const icep_params &params() const override { return P; }
  int n_particles() const override { return np; }
  int charge_field_data(double *const *out) override {
    if (!electrolyte) return fail(ICEP_ERR_UNSUPPORTED, "charge field output needs the electrolyte model");
    const int U0 = F_KR, U1 = F_KR0, U2 = F_KP, PHI = F_KV, SURF = F_KS, C0 = F_KT, C1 = F_KY, SOL = F_KZ;
    zeta_k2u_k<R>(g, f[F_ZETA0], f[F_ZETA1], ukdc, f[U0], f[U1], f[U2], s);
    c2r(f[U0], f[U1], f[U2]);
    zero(PHI);
    zero(SURF);
    scatter_profile<R>(pp, dp, dsek, f[PHI], f[SURF], PROF_QQ, s);
    sum_abs_real<R>(g, f[SURF], partials, scal, S_AUX1, s);
    int st = read_scal();
    if (st) return st;
    // 0/0 = NaN everywhere when no particle is charged, as the reference's
    const double rescale = abs_total_qe / (hscal[S_AUX1] * P.dx * P.dx * P.dx);
    scale_copy<R>(g, f[SURF], f[SURF], (R)rescale, s);
    const double area = (4. * M_PI) * (radius * radius);
    scale_copy<R>(g, f[SURF], f[SURF], (R)area, s);
    copy(C0, F_C0);
    copy(C1, F_C1);
    c2r(f[C0], f[C1]);
    solute_charge<R>(g, f[SOL], f[C0], f[C1], f[PHI], valency_e[0], valency_e[1], s);
    const int ids[8] = {U0, U1, U2, PHI, SURF, SOL, F_POT, F_EPS};
    int sel[8];
    double *dst[8];
    int n = 0;
    for (int k = 0; k < 8; k++)
      if (out[k]) {
        sel[n] = ids[k];
        dst[n++] = out[k];
      }
    return n ? get_fields(sel, dst, n) : sync();
  }
  int set_field(int id, const double *host) override {
    if (id < 0 || id >= F_COUNT) return fail(ICEP_ERR_ARG, "field id");
    if (id == F_POT && mixed) {
      cudaMemcpyAsync(stage, host, sizeof(double) * g.nf(), cudaMemcpyHostToDevice, s);
      return import_potential(stage);
    }
    if (sizeof(R) == sizeof(double)) {
      cudaMemcpyAsync(f[id], host, sizeof(double) * g.nf(), cudaMemcpyHostToDevice, s);
    } else {
      cudaMemcpyAsync(stage, host, sizeof(double) * g.nf(), cudaMemcpyHostToDevice, s);
      convert_d2f(g.nf(), stage, (float *)f[id], s);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("set_field");
    return ICEP_OK;
  }
  // ---- checkpoint / restart (Save_Restart_udf / Force_restore_parameters,
  // resume.cxx:10-78, 308-398, plus the potential) -----------------------
  // Binary, host byte order:
  //   "ICEPCKP1", int32 nx ny nz n_particles precision electrolyte nfield spec
  //   int64 ts, double time, double uk_dc[3]
  //   nfield x (int32 field id, NX*NY*NZ_ doubles)
  //   n_particles x icep_particle
  //   spec != 0: int32 xp_valid, then the float-float potential spectrum and
  //   the previous one (MIXED electrolyte; NX*NY*NZ_ x 8 bytes each)
  // FP32 fields are stored as doubles (exact both ways).
  static constexpr char CKPT_MAGIC[9] = "ICEPCKP1";
  void ckpt_fields(int *ids, int *n) const {
    *n = 0;
    ids[(*n)++] = F_ZETA0;
    ids[(*n)++] = F_ZETA1;
    if (electrolyte) {
      ids[(*n)++] = F_C0;
      ids[(*n)++] = F_C1;
      ids[(*n)++] = F_POT;
    }
  }
  int save_checkpoint(const char *path) override {
    if (!path) return fail(ICEP_ERR_ARG, "checkpoint path");
    int ids[8], nfld;
    ckpt_fields(ids, &nfld);
    const long nf = g.nf();
    std::vector<double> buf((size_t)nf);
    FILE *fp = fopen(path, "wb");
    if (!fp) return fail(ICEP_ERR_IO, "cannot open the checkpoint file for writing");
    const int spec = (mixed && electrolyte && x64_valid) ? 1 : 0;
    const int32_t hdr[8] = {g.nx, g.ny, g.nz, np, mixed ? ICEP_MIXED : ICEP_FP64, electrolyte ? 1 : 0, nfld, spec};
    const int64_t ts64 = ts;
    double ukh[3];
    bool okw = get_uk_dc(ukh) == ICEP_OK;
    okw = okw && fwrite(CKPT_MAGIC, 1, 8, fp) == 8 && fwrite(hdr, sizeof(hdr), 1, fp) == 1 &&
          fwrite(&ts64, sizeof(ts64), 1, fp) == 1 && fwrite(&time, sizeof(time), 1, fp) == 1 &&
          fwrite(ukh, sizeof(ukh), 1, fp) == 1;
    for (int q = 0; q < nfld && okw; q++) {
      const int32_t id = ids[q];
      if (sizeof(R) == sizeof(double)) {
        cudaMemcpyAsync(buf.data(), f[id], sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
      } else {
        convert_f2d(nf, (const float *)f[id], stage, s);
        cudaMemcpyAsync(buf.data(), stage, sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
      }
      okw = cudaStreamSynchronize(s) == cudaSuccess && fwrite(&id, sizeof(id), 1, fp) == 1 &&
            fwrite(buf.data(), sizeof(double), (size_t)nf, fp) == (size_t)nf;
    }
    if (okw && np > 0) {
      cudaMemcpyAsync(hp, dp, sizeof(icep_particle) * np, cudaMemcpyDeviceToHost, s);
      okw = cudaStreamSynchronize(s) == cudaSuccess && fwrite(hp, sizeof(icep_particle), (size_t)np, fp) == (size_t)np;
    }
    if (okw && spec) {
      const int32_t xpv = xp_valid ? 1 : 0;
      okw = fwrite(&xpv, sizeof(xpv), 1, fp) == 1;
      const int ds[2] = {D_X, D_XP};
      for (int q = 0; q < 2 && okw; q++) {
        cudaMemcpyAsync(buf.data(), d64[ds[q]], sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
        okw = cudaStreamSynchronize(s) == cudaSuccess &&
              fwrite(buf.data(), sizeof(double), (size_t)nf, fp) == (size_t)nf;
      }
    }
    if (fclose(fp) != 0) okw = false;
    if (!okw) return fail(ICEP_ERR_IO, "writing the checkpoint failed");
    return cuda_status("save_checkpoint");
  }
  int load_checkpoint(const char *path) override {
    if (!path) return fail(ICEP_ERR_ARG, "checkpoint path");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(ICEP_ERR_IO, "cannot open the checkpoint file");
    const long nf = g.nf();
    char magic[8];
    int32_t hdr[8];
    int64_t ts64 = 0;
    double tm = 0.0, ukh[3];
    int st = ICEP_OK;
    std::string why;
    if (fread(magic, 1, 8, fp) != 8 || memcmp(magic, CKPT_MAGIC, 8) != 0 || fread(hdr, sizeof(hdr), 1, fp) != 1 ||
        fread(&ts64, sizeof(ts64), 1, fp) != 1 || fread(&tm, sizeof(tm), 1, fp) != 1 ||
        fread(ukh, sizeof(ukh), 1, fp) != 1) {
      st = ICEP_ERR_IO;
      why = "not a checkpoint file or truncated header";
    } else if (hdr[0] != g.nx || hdr[1] != g.ny || hdr[2] != g.nz || hdr[3] != np ||
               hdr[4] != (mixed ? ICEP_MIXED : ICEP_FP64) || hdr[5] != (electrolyte ? 1 : 0) || hdr[6] < 0 ||
               hdr[6] > 8 || hdr[7] < 0 || hdr[7] > 1) {
      st = ICEP_ERR_ARG;
      why = "checkpoint does not match the context (mesh, particle count, precision or model)";
    }
    // read everything into host memory first: a failed load leaves the context unchanged
    std::vector<int32_t> ids;
    std::vector<double> data;
    std::vector<icep_particle> parts;
    std::vector<double> spec;
    int32_t xpv = 0;
    if (st == ICEP_OK) {
      ids.resize((size_t)hdr[6]);
      data.resize((size_t)hdr[6] * (size_t)nf);
      for (int q = 0; q < hdr[6] && st == ICEP_OK; q++) {
        if (fread(&ids[q], sizeof(int32_t), 1, fp) != 1 ||
            fread(data.data() + (size_t)q * nf, sizeof(double), (size_t)nf, fp) != (size_t)nf) {
          st = ICEP_ERR_IO;
          why = "truncated checkpoint (fields)";
        } else if (ids[q] < 0 || ids[q] >= F_COUNT) {
          st = ICEP_ERR_ARG;
          why = "checkpoint field id out of range";
        }
      }
      parts.resize((size_t)(np > 0 ? np : 1));
      if (st == ICEP_OK && np > 0 && fread(parts.data(), sizeof(icep_particle), (size_t)np, fp) != (size_t)np) {
        st = ICEP_ERR_IO;
        why = "truncated checkpoint (particles)";
      }
      if (st == ICEP_OK && hdr[7]) {
        spec.resize(2 * (size_t)nf);
        if (fread(&xpv, sizeof(xpv), 1, fp) != 1 ||
            fread(spec.data(), sizeof(double), 2 * (size_t)nf, fp) != 2 * (size_t)nf) {
          st = ICEP_ERR_IO;
          why = "truncated checkpoint (potential spectrum)";
        }
      }
    }
    fclose(fp);
    if (st != ICEP_OK) return fail(st, why.c_str());
    if ((st = set_particles(parts.data())) != ICEP_OK) return st;
    for (size_t q = 0; q < ids.size(); q++)
      if ((st = set_field(ids[q], data.data() + q * nf)) != ICEP_OK) return st;
    if ((st = set_uk_dc(ukh)) != ICEP_OK) return st;
    pot_export_valid = false;
    if (hdr[7]) {  // after set_field(F_POT), which invalidates the spectrum
      cudaMemcpyAsync(d64[D_X], spec.data(), sizeof(double) * nf, cudaMemcpyHostToDevice, s);
      cudaMemcpyAsync(d64[D_XP], spec.data() + nf, sizeof(double) * nf, cudaMemcpyHostToDevice, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("load_checkpoint");
      x64_valid = true;
      xp_valid = xpv != 0;
    }
    ts = (int)ts64;
    time = tm;
    return ICEP_OK;
  }
  int get_particles(icep_particle *h) override {
    cudaMemcpyAsync(hp, dp, sizeof(icep_particle) * np, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("get_particles");
    memcpy(h, hp, sizeof(icep_particle) * np);
    return ICEP_OK;
  }
  int set_particles(const icep_particle *h) override {
    const int st = put_particles(h);
    if (st) return st;
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("set_particles");
    return ICEP_OK;
  }
  // set_particles without the final synchronisation (the copy from the
  // pinned staging array queued)
  int put_particles(const icep_particle *h) {
    // species in range; the field stays Janus (every species with an axis) or
    // not (particle 0's species without one), as the context was created
    for (int q = 0; q < np; q++) {
      if (h[q].spec < 0 || h[q].spec >= P.n_species) return fail(ICEP_ERR_ARG, "particle species out of range");
      const bool ax = P.janus_axis[h[q].spec] != ICEP_JANUS_NONE;
      if ((janus && !ax) || (!janus && q == 0 && ax))
        return fail(ICEP_ERR_ARG, "set_particles: species Janus axes do not match the context's permittivity field");
    }
    cudaStreamSynchronize(s);
    memcpy(hp, h, sizeof(icep_particle) * np);
    if (!P.per_particle_eps)
      for (int q = 0; q < np; q++) hp[q].eps_p = P.eps_particle_top;
    cudaMemcpyAsync(dp, hp, sizeof(icep_particle) * np, cudaMemcpyHostToDevice, s);
    return ICEP_OK;
  }
  int get_uk_dc(double *v) override {
    double tmp[3];
    cudaMemcpyAsync(tmp, ukdc, sizeof(tmp), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int d = 0; d < 3; d++) v[d] = tmp[d];
    return cuda_status("get_uk_dc");
  }
  int set_uk_dc(const double *v) override {
    cudaMemcpyAsync(ukdc, v, sizeof(double) * 3, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    return cuda_status("set_uk_dc");
  }
  int fft_host(double *a, bool forward) override {
    int st = set_field(F_WORK, a);
    if (st) return st;
    if (forward) r2c(f[F_WORK]);
    else c2r(f[F_WORK]);
    return get_field(F_WORK, a);
  }
  int apply_A_host(const double *x, double *y) override {
    std::vector<double> pad(g.nf(), 0.0);
    for (long ij = 0; ij < (long)g.nx * g.ny; ij++)
      memcpy(&pad[ij * g.nzp], x + ij * g.nz, sizeof(double) * g.nz);
    int st = set_field(F_KP, pad.data());
    if (st) return st;
    apply_A(f[F_KP], f[F_KV]);
    if ((st = get_field(F_KV, pad.data()))) return st;
    for (long ij = 0; ij < (long)g.nx * g.ny; ij++)
      memcpy(y + ij * g.nz, &pad[ij * g.nzp], sizeof(double) * g.nz);
    return ICEP_OK;
  }
  int lj_pairs(int *pairs, int max_pairs, int *n) override {
    int *dpairs = nullptr;
    if (max_pairs > 0 && cudaMalloc(&dpairs, sizeof(int) * 2 * max_pairs) != cudaSuccess)
      return fail(ICEP_ERR_CUDA, "cudaMalloc pairs");
    cudaMemsetAsync(dpairs_n, 0, sizeof(int), s);
    // the pair scan accumulates into fr: clear it first, as the harness does
    cudaMemcpyAsync(hp, dp, sizeof(icep_particle) * np, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int q = 0; q < np; q++)
      for (int d = 0; d < 3; d++) hp[q].fr[d] = 0.0;
    cudaMemcpyAsync(dp, hp, sizeof(icep_particle) * np, cudaMemcpyHostToDevice, s);
    int st = lj_force(pp, dp, ljwork, ljwork_ints, dpairs, max_pairs, dpairs_n, s);
    if (st) {
      cudaFree(dpairs);
      return fail(st, "LJ cell list");
    }
    cudaMemcpyAsync(n, dpairs_n, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    const int m = (*n < max_pairs) ? *n : max_pairs;
    if (m > 0) cudaMemcpyAsync(pairs, dpairs, sizeof(int) * 2 * m, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFree(dpairs);
    return cuda_status("lj_pairs");
  }
  int time_kernel(int which, int nb, int reps, double *ms, double *bytes) override {
    if (nb < 1 || nb > 5 || reps < 1) return fail(ICEP_ERR_ARG, "time_kernel arguments");
    const int ids[5] = {F_WV3_0, F_WV3_1, F_WV3_2, F_KY, F_KZ};
    FieldBatch<R> fb = batch(f[ids[0]], nb > 1 ? f[ids[1]] : nullptr, nb > 2 ? f[ids[2]] : nullptr,
                             nb > 3 ? f[ids[3]] : nullptr, nb > 4 ? f[ids[4]] : nullptr);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto one = [&]() {
      if (which <= 3) fft_pass(fft, fb, which, s);
      else if (which == 7) fft_r2c(fft, fb, s);
      else if (which == 8) fft_c2r(fft, fb, s);
      else if (which == 10 && mixed && d64[D_X]) residual_df(1.f);
      else apply_A(f[F_KP], f[F_KV]);
    };
    one();  // warm-up
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps; r++) one();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = (double)t / reps;
    const double field = (double)g.nreal() * sizeof(R);
    if (which <= 8) *bytes = 2.0 * field * nb;  // one field in, one out, per transform or pass
    else if (which == 10) *bytes = 17.0 * (double)g.nreal() * sizeof(double);
    else *bytes = 17.0 * field;                      // Ax: 8 FFTs + the permittivity read
    return cuda_status("time_kernel");
  }

  int phase_times(double *ms, int n) override {
    for (int k = 0; k < n && k < NPH; k++) ms[k] = ph_ms[k];
    return phase_on ? ICEP_OK : ICEP_ERR_STATE;
  }

  int tile_picks(int *picks, double *us) override {
    if (!kop_tuned) return fail(ICEP_ERR_STATE, "no tuned fused passes in this context (MIXED electrolyte, NX <= 128)");
    picks[0] = kop_tiles.xinv_kw;
    picks[1] = kop_tiles.xfwd_kw;
    picks[2] = kop_tiles.plane_smem;
    if (us)
      for (int k = 0; k < 8; k++) us[k] = kop_tune_us[k];
    return ICEP_OK;
  }

  int selftest_wait(int kernel) override {
    if constexpr (std::is_same<R, float>::value) {
      int *word = nullptr;
      if (kernel == 1) {
        word = kerr;
        cudaMemsetAsync(word, 0, sizeof(int), s);
        if (!kop_plane_selftest(fft, f[F_WV3_0], f[F_WV3_1], f[F_WV3_2], f[F_WV3_3], f[F_EF0], f[F_EF1], f[F_EF2], word, s))
          return fail(ICEP_ERR_UNSUPPORTED, "wait self-test: no register plane kernel for this mesh");
      } else if (kernel == 2 && learned) {
        word = net.err;
        cudaMemsetAsync(word, 0, sizeof(int), s);
        net.selftest_wait(s);
      } else {
        return EngineBase::selftest_wait(kernel);
      }
      int h = 0;
      cudaMemcpyAsync(&h, word, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("wait self-test");
      cudaMemsetAsync(word, 0, sizeof(int), s);  // re-armed for the next solve
      if (h) return fail(ICEP_ERR_TIMEOUT, kernel == 1 ? "fused plane pass: bounded wait ran out (self-test)"
                                                        : "network convolution: bounded wait ran out (self-test)");
      return ICEP_OK;
    } else {
      return EngineBase::selftest_wait(kernel);
    }
  }

  int sync() override {
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("sync");
    return ICEP_OK;
  }

  int call(int fn) override {
    int st = ICEP_OK;
    switch (fn) {
      case C_ZETA_K2U_K:
        zeta_k2u_k<R>(g, f[F_ZETA0], f[F_ZETA1], ukdc, f[F_U0], f[F_U1], f[F_U2], s);
        break;
      case C_ZETA_K2U: zeta_k2u(); break;
      case C_U_K2ZETA_K:
        u_k2zeta_k<R>(g, f[F_U0], f[F_U1], f[F_U2], f[F_ZETA0], f[F_ZETA1], ukdc, s);
        break;
      case C_U2ADVECTION_K: u2advection_k(F_NS0_0, F_NS0_1); break;
      case C_SOLENOIDAL_U: solenoidal_u(F_U0); break;
      case C_NS_SLAVED_EULER: ns_solver_slaved_euler(); break;
      case C_MAKE_PHI_SUM: make_phi_particle_sum(); break;
      case C_MAKE_U_SUM: make_u_particle_sum(); break;
      case C_F_HYDRO: f_hydro<R>(pp, dp, dsek, f[F_PHI_SUM], f[F_U0], f[F_U1], f[F_U2], false, s); break;
      case C_LJ: {
        int n = 0;
        st = lj_pairs(nullptr, 0, &n);
        break;
      }
      case C_POS_EULER: md_position(pp, dp, false, s); break;
      case C_POS_AB2: md_position(pp, dp, true, s); break;
      case C_VEL_EULER:
      case C_VEL_AB2:
        if ((st = lj_into_fr())) break;
        md_velocity(pp, dp, fn == C_VEL_AB2, s);
        break;
      case C_DIELECTRIC_FIELD: make_dielectric_field(F_WORK, F_WV1); break;
      case C_BUILD_RHS: build_rhs(F_WORK, F_RHO); break;
      case C_SOLVE_POTENTIAL: st = solve_potential(F_RHO, F_POT, F_WORK); break;
      case C_MAXWELL: st = maxwell_force(F_RHO); break;
      case C_NSSOLUTE_EULER: nssolute_solver_euler(); break;
      case C_SURFACE_NORMAL:
        for (int d = 0; d < 3; d++) zero(F_SN0 + d);
        scatter_normal<R>(pp, dp, dsek, f[F_SN0], f[F_SN1], f[F_SN2], s);
        break;
      case C_F_PARTICLE_SOLE:
        f_nonsole<R>(g, vec(F_F0), vec(F_UP0), f[F_PHI], vec(F_U0), s);
        solenoidal_u(F_F0);
        break;
      case C_TRUNCATE: truncate_23<R>(g, batch(f[F_ZETA0], f[F_ZETA1]), s); break;
      case C_CHARGE_FIELD: st = conc_k2charge(F_RHO, F_WORK, F_UP0); break;
      case C_INIT_ION: st = init_ions(); break;
      case C_APPLY_BK:
        if constexpr (std::is_same<R, float>::value) {
          if (!kop_supported(g)) return fail(ICEP_ERR_UNSUPPORTED, "apply_bk: no fused passes for this mesh");
          mean_eps_cached = mean_eps();
          kop_eps_faces(g, f[F_EPS], f[F_EF0], f[F_EF1], f[F_EF2], s);
          apply_Bk(f[F_WV1], f[F_WORK]);
          break;
        } else {
          return fail(ICEP_ERR_UNSUPPORTED, "apply_bk needs precision MIXED");
        }
      default: return fail(ICEP_ERR_ARG, "unknown call id");
    }
    if (st) return st;
    if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status("call");
    return cuda_status("call");
  }
};

}  // namespace

EngineBase *make_engine(const icep_params &p, const icep_particle *parts, int np, int *status, std::string &err) {
  EngineBase *e = nullptr;
  int st;
  if (p.precision == ICEP_MIXED) {
    auto *m = new Engine<float>();
    st = m->setup(p, parts, np);
    e = m;
  } else {
    auto *m = new Engine<double>();
    st = m->setup(p, parts, np);
    e = m;
  }
  if (st != ICEP_OK) {
    err = e->err;
    delete e;
    e = nullptr;
  }
  if (status) *status = st;
  return e;
}

}  // namespace icep
