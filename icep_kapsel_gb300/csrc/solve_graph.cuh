// solve_graph.cuh -- the MIXED Poisson solve's control on the device, for
// steps captured whole as one CUDA graph (no counterpart in the reference,
// whose Charge_field2potential_dielectric, operate_dielectric.cxx:542-572,
// loops on the host).
//
// The refinement sweeps and the inner fused BiCGSTAB iterations become
// conditional WHILE nodes. Each loop body ends with a one-block kernel that
// takes the decision the host loop takes, in the same double arithmetic, and
// sets the loop's condition; the scalars the host loop passes as kernel
// arguments (the residual prescale, 1/|r|, |r|, 1/eps_ref) live in a small
// device array instead. Every loop is bounded: the inner loop by the
// iteration limit (enforced by kop_xr and, as a guard, by the body count),
// the sweeps by 30.
#pragma once
#include <vector>

#include "common.cuh"

namespace icep {

// A refinement sweep's inner tolerance: INNER_MARGIN tol |b| / |r| (clamped
// to [2e-5, 0.5]), so that the sweep's true residual lands below tol with
// room for the FP32 solve's deviation from it. Measured on GB300 at 128^3
// (40 steps of the 512-sphere workload): margin 0.5 / 0.6 / 0.7 / 0.8 ->
// 17.05 / 16.08 / 15.26 / 15.05 inner iterations per step, largest true
// residual 4.9e-9 / 5.8e-9 / 7.0e-9 / 7.7e-9 at tol 1e-8, one sweep every
// step; a sweep that misses tol is followed by another.
constexpr double INNER_MARGIN = 0.7;

// doubles of the control array
enum {
  SC_BB = 0,     // |b^|^2 / N of the right-hand side
  SC_TOL2,       // tol^2 SC_BB
  SC_ZERO_RHS,   // 1: b = 0 (x = 0, no sweep)
  SC_STATUS,     // ICEP_OK, or the error code of a non-finite value
  SC_SWEEPS,     // correction sweeps started
  SC_INNER,      // inner iterations over the finished sweeps
  SC_REL,        // |r| / |b| of the last true residual
  SC_INNER_TOL,  // the current sweep's inner tolerance
  SC_LOOPS,      // inner loop bodies run in the current sweep
  SC_GUARD,      // 1: a loop stopped on its body-count guard
  SC_COUNT
};
// floats of the control array (8-byte aligned): the residual prescale, 1/|r|
// of the sweep's normalisation and |r| as a float-float pair (hi, lo)
enum { SCF_PRESCALE = 0, SCF_INVRN, SCF_RN, SCF_COUNT = 4 };

// After the right-hand side: SC_BB, SC_TOL2, SC_ZERO_RHS, the prescale and
// ks[KS_IEPS] = 1/eps_ref from scal[slot_bb] (|b^|^2/N) and scal[slot_eps]
// (the sum of eps over the real points); the counters reset.
void solve_begin(const double *scal, int slot_bb, int slot_eps, double *sc, float *scf, double *ks, double tol,
                 double nreal, cudaStream_t s);
// After each true residual (|r^|^2/N in scal[slot_rr]): the sweep loop's
// condition. add_inner: the finished sweep's iterations (ks[KS_ITERS]) are
// added first. For a further sweep: 1/|r|, |r| and the inner tolerance.
void sweep_cond(cudaGraphConditionalHandle h, const double *scal, int slot_rr, double *sc, float *scf,
                const double *ks, double tol, double nreal, int max_sweeps, bool add_inner, cudaStream_t s);
// After |r|^2 of the sweep's normalised residual (scal[slot_rr]): the inner
// iteration's starting state in ks (BiCGSTAB, or with cg the preconditioned
// CG) and the inner loop's condition.
void inner_prep(cudaGraphConditionalHandle h, const double *scal, int slot_rr, double *sc, double *ks, double eps2,
                bool cg, cudaStream_t s);
// End of a BiCGSTAB inner loop body: a restart that kop_xr asked for (r0 =
// r, v = p = 0, the scalars reset) or the stop, as the host loop does it; nf
// floats per vector. (A CG body needs no such kernel: kop_cg's last block
// sets the loop's condition.)
void inner_cond(cudaGraphConditionalHandle h, double *ks, float *r, float *r0, float *v, float *p, long nf,
                int maxit, double *sc, double eps2, cudaStream_t s);

// ---- graph building by stream capture ------------------------------------
// Stream work appended to graph `gr` after the nodes `deps`; `leaf` receives
// the nodes that end what was appended (deps itself when nothing was).
inline cudaError_t cap_begin(cudaStream_t s, cudaGraph_t gr, const std::vector<cudaGraphNode_t> &deps) {
  return cudaStreamBeginCaptureToGraph(s, gr, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                       cudaStreamCaptureModeThreadLocal);
}
inline cudaError_t cap_end(cudaStream_t s, std::vector<cudaGraphNode_t> &leaf) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  const cudaGraphNode_t *d = nullptr;
  size_t n = 0;
  const cudaError_t e = cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &d, nullptr, &n);
  if (e == cudaSuccess) leaf.assign(d, d + n);
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(s, &g);
  return e != cudaSuccess ? e : e2;
}
// A WHILE node in `gr` after `deps` on the handle h (created on gr with
// cudaGraphConditionalHandleCreate, value 0 at each launch: a kernel before
// the node sets it) and its body graph.
inline cudaError_t add_while(cudaGraph_t gr, const std::vector<cudaGraphNode_t> &deps, cudaGraphConditionalHandle h,
                             cudaGraphNode_t *node, cudaGraph_t *body) {
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  const cudaError_t e = cudaGraphAddNode(node, gr, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &p);
  if (e != cudaSuccess) return e;
  *body = p.conditional.phGraph_out[0];
  return cudaSuccess;
}

}  // namespace icep
