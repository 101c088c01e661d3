// solve_graph.cu -- device-side control of the MIXED Poisson solve (see
// solve_graph.cuh). The decisions follow the host loop of the engine's
// solve_potential_mixed and bicgstab_kf line by line, in the same double
// arithmetic, so that a step run as one graph computes what the host-driven
// step computes.
#include <cfloat>

#include "kop.cuh"
#include "solve_graph.cuh"

namespace icep {

namespace {

__global__ void k_solve_begin(const double *scal, int slot_bb, int slot_eps, double *sc, float *scf, double *ks,
                              double tol, double nreal) {
  const double bb = scal[slot_bb];
  sc[SC_BB] = bb;
  sc[SC_TOL2] = tol * tol * bb;
  sc[SC_STATUS] = isfinite(bb) ? (double)ICEP_OK : (double)ICEP_ERR_NOT_CONVERGED;
  const bool zero = !(bb > 0.0);
  sc[SC_ZERO_RHS] = zero ? 1.0 : 0.0;
  // squares summed in FP32 after a power-of-two prescale that brings
  // sum_k |b^_k|^2 to order 1, the exponent kept inside FP32's range
  float prescale = 1.f;
  if (!zero && isfinite(bb)) {
    int pe = -ilogb(sqrt(nreal * bb));
    pe = pe < -100 ? -100 : pe > 100 ? 100 : pe;
    prescale = (float)ldexp(1.0, pe);
  }
  scf[SCF_PRESCALE] = prescale;
  ks[KS_IEPS] = 1.0 / (scal[slot_eps] / nreal);
  sc[SC_SWEEPS] = 0.0;
  sc[SC_INNER] = 0.0;
  sc[SC_REL] = 0.0;
  sc[SC_GUARD] = 0.0;
}

__global__ void k_sweep_cond(cudaGraphConditionalHandle h, const double *scal, int slot_rr, double *sc, float *scf,
                             const double *ks, double tol, double nreal, int max_sweeps, int add_inner) {
  if (add_inner) sc[SC_INNER] += ks[KS_ITERS];
  unsigned go = 0;
  const double rr = scal[slot_rr];
  if (sc[SC_ZERO_RHS] != 0.0 || sc[SC_STATUS] != (double)ICEP_OK) {
    // b = 0 (x is set to zero after the loop) or a non-finite b
  } else {
    sc[SC_REL] = sqrt(rr / sc[SC_BB]);
    if (!isfinite(rr)) {
      sc[SC_STATUS] = (double)ICEP_ERR_NOT_CONVERGED;
    } else if (rr > sc[SC_TOL2] && sc[SC_SWEEPS] < (double)max_sweeps) {
      // FP32 correction solve on the normalised residual
      const double rn = sqrt(rr / nreal);
      scf[SCF_INVRN] = (float)(1.0 / rn);
      const float hi = (float)rn;
      scf[SCF_RN] = hi;
      scf[SCF_RN + 1] = (float)(rn - (double)hi);
      double inner_tol = INNER_MARGIN * tol * sqrt(sc[SC_BB] / rr);
      if (inner_tol < 2e-5) inner_tol = 2e-5;
      if (inner_tol > 0.5) inner_tol = 0.5;
      sc[SC_INNER_TOL] = inner_tol;
      sc[SC_SWEEPS] += 1.0;
      go = 1;
    }
  }
  cudaGraphSetConditional(h, go);
}

__global__ void k_inner_prep(cudaGraphConditionalHandle h, const double *scal, int slot_rr, double *sc, double *ks,
                             double eps2, int cg) {
  const double bsq = scal[slot_rr];
  sc[SC_LOOPS] = 0.0;
  ks[KS_ITERS] = 0.0;
  if (!(bsq > 0.0)) {  // the correction is zero
    ks[KS_DONE] = 1.0;
    cudaGraphSetConditional(h, 0u);
    return;
  }
  const double tol = sc[SC_INNER_TOL];
  // BiCGSTAB iteration 0: rho = (r0, r), p = v = 0; CG: p = r (beta = 0,
  // omega = 0), rho formed by kop_cg's starting pass
  ks[KS_RHO] = bsq;
  ks[KS_BETA] = cg ? 0.0 : 1.0;
  ks[KS_OMEGA] = cg ? 0.0 : 1.0;
  ks[KS_TOL2] = tol * tol * bsq;
  ks[KS_DONE] = 0.0;
  ks[KS_RR] = bsq;
  ks[KS_RESTART] = cg ? 0.0 : eps2 * bsq;
  cudaGraphSetConditional(h, bsq > ks[KS_TOL2] ? 1u : 0u);
}

// one block: the restart's vector work (rare) is block-strided
__global__ void __launch_bounds__(1024) k_inner_cond(cudaGraphConditionalHandle h, double *ks, float *r, float *r0,
                                                     float *v, float *p, long nf, int maxit, double *sc, double eps2) {
  __shared__ double done;
  if (threadIdx.x == 0) done = ks[KS_DONE];
  __syncthreads();
  if (done == 2.0) {  // restart on the current residual
    for (long q = threadIdx.x; q < nf; q += blockDim.x) {
      r0[q] = r[q];
      v[q] = 0.f;
      p[q] = 0.f;
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double loops = sc[SC_LOOPS] + 1.0;
  sc[SC_LOOPS] = loops;
  unsigned go = 1;
  if (done == 1.0) {
    go = 0;
  } else if (loops > (double)maxit + 2.0) {  // guard: kop_xr stops at maxit
    sc[SC_GUARD] = 1.0;
    go = 0;
  } else if (done == 2.0) {
    const double rr = ks[KS_RR];
    if (!(rr > 0.0)) {
      go = 0;
    } else {
      ks[KS_RHO] = rr;
      ks[KS_BETA] = 1.0;
      ks[KS_OMEGA] = 1.0;
      ks[KS_RESTART] = eps2 * rr;
      ks[KS_DONE] = 0.0;
    }
  }
  cudaGraphSetConditional(h, go);
}

}  // namespace

void solve_begin(const double *scal, int slot_bb, int slot_eps, double *sc, float *scf, double *ks, double tol,
                 double nreal, cudaStream_t s) {
  count_launch();
  k_solve_begin<<<1, 1, 0, s>>>(scal, slot_bb, slot_eps, sc, scf, ks, tol, nreal);
}
void sweep_cond(cudaGraphConditionalHandle h, const double *scal, int slot_rr, double *sc, float *scf,
                const double *ks, double tol, double nreal, int max_sweeps, bool add_inner, cudaStream_t s) {
  count_launch();
  k_sweep_cond<<<1, 1, 0, s>>>(h, scal, slot_rr, sc, scf, ks, tol, nreal, max_sweeps, add_inner ? 1 : 0);
}
void inner_prep(cudaGraphConditionalHandle h, const double *scal, int slot_rr, double *sc, double *ks, double eps2,
                bool cg, cudaStream_t s) {
  count_launch();
  k_inner_prep<<<1, 1, 0, s>>>(h, scal, slot_rr, sc, ks, eps2, cg ? 1 : 0);
}
void inner_cond(cudaGraphConditionalHandle h, double *ks, float *r, float *r0, float *v, float *p, long nf,
                int maxit, double *sc, double eps2, cudaStream_t s) {
  count_launch();
  k_inner_cond<<<1, 1024, 0, s>>>(h, ks, r, r0, v, p, nf, maxit, sc, eps2);
}

}  // namespace icep
