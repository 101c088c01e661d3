// kop.cuh -- the k-space Poisson iteration's operator B = A M^-1 fused into
// three FFT passes, with the BiCGSTAB vector updates and dot products folded
// into them (FP32, the inner solver of MIXED precision).
//
//   kop_xinv : vector update (p or s) at the read modes, then the inverse x
//              transforms of the x gradient m(k) i k_x exp(i dx k_x/2) p into
//              w0 and of M = m(k) p into w1 (the y and z gradient multipliers
//              depend on (j, kz) only and commute with the x transform)
//   kop_plane: per x-plane and component d: the y or z gradient factor on M
//              (d = 1, 2), inverse y/z transform, multiplication by the face
//              permittivity eps_face_d (the reference's 0.5 (eps + eps
//              shifted along d), operate_dielectric.cxx:485-522), forward z/y
//              transform, the divergence factor k_d exp(-i dx k_d/2) (d = 1,
//              2) -- into w0 (d = 0, in place), w2 and w3; the real field
//              never leaves shared memory
//   kop_xfwd : forward x transforms of w0 (times k_x exp(-i dx k_x/2)) and of
//              w2 + w3, their sum times i into the output vector (the
//              staggered divergence), with the dot products the iteration
//              needs next as per-block partials
//   (Planes too large for one block take the split plane step: kop_xinv
//   writes the three gradients, the plain y/z passes transform them around
//   the product, and kop_xfwd takes the three divergence factors.)
//   kop_xr   : x~ += alpha p + omega s, r = s - omega t and the dot products
//              (r0, r), (r, r)
// Vectors follow kspace.cuh (read modes only). Dot partials are FP64, one or
// two per block, scaled by 1/N; the last block of a pass sums them in a fixed
// order into two final numbers.
#pragma once
#include "fft.cuh"

namespace icep {

enum { KOP_P = 0, KOP_S = 1, KOP_NONE = 2, KOP_CG = 3, KOP_PC = 4 };

// true if the fused passes cover this grid (an x-plane fits in shared memory)
bool kop_supported(const Grid &g);
// The plane pass of the plain FP32 3D transforms (fft.cuh) by the
// register-resident kernels (C2R with `inverse`, else R2C) when the plan has
// an error word (p.err) and the plane has a register kernel (NY in {64, 128},
// NZ/2 in {32, 64}, NZ/2 <= NY); false (nothing launched) otherwise.
bool fft_plane_r(const FFTPlan<float> &p, const FieldBatch<float> &fb, bool inverse, cudaStream_t s);

// Tile choices of the fused passes: x pencils per block of the inverse and
// forward x passes (8, 16 or 32 for NX in {64, 128}; 16 otherwise), and the
// plane pass's implementation (0: the register-resident kernel where the
// mesh has one, 1: the shared-memory kernel).
struct KopTiles {
  int xinv_kw = 16, xfwd_kw = 16, plane_smem = 0;
};
// The tile autotuner: times every candidate of each pass (5 launches each
// after one warm-up, CUDA events on s) on the given scratch fields -- any
// values: the operator runs without vector update or dots -- and returns the
// faster plane kernel and, per x pass, the default 16 pencils unless a
// candidate is more than 3% faster (then the fastest); `us` (optional, 8
// values) receives the times per launch in the
// order xinv 8/16/32, xfwd 8/16/32, plane register/shared (0 where a
// candidate does not exist for the mesh). The picks are cached per mesh for
// the process, so later contexts of the same mesh take them untimed.
KopTiles kop_autotune(const FFTPlan<float> &p, float *vec, float *w0, float *w1, float *w2, float *w3,
                      const float *ef0, const float *ef1, const float *ef2, float *out, int *err, cudaStream_t s,
                      double *us);
// Device-side BiCGSTAB iteration state (doubles). With a state pointer
// kop_xinv takes beta, omega and rho from it instead of its arguments, and
// kop_xr returns without touching x and r once KS_DONE is set (the other
// passes of an iteration enqueued past the stop only write scratch vectors);
// kop_xr's last block forms the next iteration's scalars from the final sums
// and sets KS_DONE (1: converged, non-finite or at the iteration limit; 2: a
// restart for the host). The host then enqueues several iterations between
// synchronisations.
// KS_IEPS: 1/eps_ref of the solve's preconditioner (read by kop_xinv in place
// of its argument when a state pointer is given).
enum { KS_RHO = 0, KS_BETA, KS_OMEGA, KS_TOL2, KS_DONE, KS_ITERS, KS_RR, KS_RESTART, KS_IEPS, KS_COUNT };
// an upper bound on the x-pencil blocks (= partial sums written by kop_xfwd)
int kop_pencil_blocks(const Grid &g);
// ef_d = 0.5 (eps + eps at the next point along d), real points
void kop_eps_faces(const Grid &g, const float *eps, float *ef0, float *ef1, float *ef2, cudaStream_t s);
// mode KOP_P: vec = p <- P(r) + beta (P(p) - omega P(v));
// mode KOP_S: vec = s <- P(r) - alpha P(v), alpha = rho / fin[0];
// mode KOP_PC (the CG): vec = p~ <- P(r) + beta P(p~) (v unused);
// mode KOP_NONE: vec is used as it is (r, v, fin unused).
// Outputs: the x gradient into w0 and M into w1; on a mesh that takes the
// split plane step (kop_plane_fits false) the y and z gradients into w2 and
// w3 instead of M (the generic passes there take no factors).
void kop_xinv(const FFTPlan<float> &p, int mode, float *vec, const float *r, const float *v, double beta,
              double omega, double rho, const double *fin, double eps_ref, float *w0, float *w1, float *w2,
              float *w3, cudaStream_t s, const double *ks = nullptr, const KopTiles &t = KopTiles());
// err: device word set to 1 if a bulk copy into shared memory did not
// complete within the kernel's wait limit (checked by the caller)
void kop_plane(const FFTPlan<float> &p, float *w0, float *w1, float *w2, float *w3, const float *ef0,
               const float *ef1, const float *ef2, int *err, cudaStream_t s, const KopTiles &t = KopTiles());
// Bounded-wait self-test of the plane pass: the register plane kernel
// launched so that its copy-arrival wait runs out (no copy is issued), which
// sets *err; false when the grid has no register plane kernel.
bool kop_plane_selftest(const FFTPlan<float> &p, float *w0, float *w1, float *w2, float *w3, const float *ef0,
                        const float *ef1, const float *ef2, int *err, cudaStream_t s);
// mode KOP_P: partials[2b] = (other, out) with other = r0;
// mode KOP_S: partials[2b] = (out, out), partials[2b+1] = (out, other) with other = s;
// finals[c] = sum over blocks of partials[2b + c], summed by the last block
// to finish (counter: a device word at zero, left at zero);
// mode KOP_CG: partials[2b] = (M^-1 other, out) = sum m(k) other^* out with
// the preconditioner m(k) (1/eps_ref from ks[KS_IEPS]): the CG denominator;
// mode KOP_NONE: no dot products (other, partials, finals unused).
void kop_xfwd(const FFTPlan<float> &p, const float *w0, const float *wa, const float *wb, float *out, int mode,
              const float *other, double *partials, double *finals, unsigned *counter, cudaStream_t s,
              const KopTiles &t = KopTiles(), const double *ks = nullptr);
// alpha = rho / fin1[0]; omega = fin2[1] / fin2[0];
// part3[2b] = (r0, r), part3[2b+1] = (r, r) over kop_xr_blocks(g) blocks,
// fin3 their sums (counter3 as for kop_xfwd).
int kop_xr_blocks(const Grid &g);
void kop_xr(const Grid &g, float *xt, float *r, const float *p, const float *sv, const float *t, const float *r0,
            double rho, const double *fin1, const double *fin2, double *part3, double *fin3, unsigned *counter3,
            cudaStream_t s, double *ks = nullptr, int maxit = 0);
// The preconditioned CG's update (the operator and preconditioner are
// symmetric): alpha = ks[KS_RHO] / fin_pq[0]; x~ += alpha p~; r -= alpha q;
// part[2b] = (r, M^-1 r), part[2b+1] = (r, r) over kop_xr_blocks(g) blocks,
// fin their sums; the last block sets KS_RHO, KS_BETA (rho'/rho, 0 with
// init), KS_OMEGA = 0, KS_ITERS, KS_RR and KS_DONE (1: converged, non-finite
// or at maxit). init: no update (the starting residual's sums only). Returns
// without touching x and r once KS_DONE is set. h (nonzero inside the step
// graph's inner WHILE loop, not with init): every launch sets the loop's
// condition, 1 while the solve is not done, 0 once it is (also when it finds
// it done on entry).
void kop_cg(const Grid &g, float *xt, float *r, const float *p, const float *q, const double *fin_pq, double *part,
            double *fin, unsigned *counter, cudaStream_t s, double *ks, int maxit, bool init,
            cudaGraphConditionalHandle h = 0);

}  // namespace icep
