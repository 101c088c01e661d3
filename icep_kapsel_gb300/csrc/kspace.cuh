// kspace.cuh -- the plain Poisson solver's Krylov iteration held in k-space.
//
// Right-preconditioned BiCGSTAB with M^-1 = -1/(eps_ref |k|^2) runs on the
// transformed vectors: B = A M^-1 is applied as
//   g_d = m(k) i k_d s_d p  ->  3 inverse FFTs  ->  * eps_face_d  ->
//   3 forward FFTs  ->  v = sum_d i k_d conj(s_d) w_d
// (s_d = exp(i dx k_d / 2), the staggered shifts of Ax in
// operate_dielectric.cxx:485-522), i.e. 6 FFTs per operator application and
// no FFT for the preconditioner. The iterate is x~ with x = x0 + M^-1 x~.
//
// The reference's inverse FFT reads only half of the kz = 0 and kz = NZ/2
// planes (the rest is implied by Hermitian symmetry) and only the real part
// at self-conjugate points. A k-space vector stands for the real field its
// inverse produces, so the kernels here read and write the read modes only
// (P(a) below: the stored entry, real part at self-conjugate points); the
// other entries are never looked at. Dot products are the real-space ones by
// Parseval over the read modes:
//   sum_r a(r) b(r) = (1/N) sum_k w(k) Re(P(a) conj(P(b))),
//   w = 1 at self-conjugate points, 2 at every other read mode.
#pragma once
#include "common.cuh"

namespace icep {

// scal[slot + c] = sum over blocks of partials[2 b + c], c < n (block order)
void kdots_finish(const double *partials, int nblocks, int n, double *scal, int slot, cudaStream_t s);
// scal[slot + c] = real-space dot of k-space vectors (a_c, b_c), c < n <= 2
template <typename R>
void kdots(const Grid &g, const R *a0, const R *b0, const R *a1, const R *b1, int n, double *partials, double *scal,
           int slot, cudaStream_t s);
// p = P(r) + beta (P(p) - w P(v))
template <typename R>
void kbicg_p(const Grid &g, R *p, const R *r, const R *v, double beta, double w, cudaStream_t s);
// s = P(r) - alpha P(v), alpha = rho / scal[S_R0V]
template <typename R>
void kbicg_s(const Grid &g, R *sv, const R *r, const R *v, double rho, const double *scal, cudaStream_t s);
// xt += alpha P(p) + w P(s); r = P(s) - w P(t), w = scal[S_TS]/scal[S_TT]
template <typename R>
void kbicg_xr(const Grid &g, R *xt, R *r, const R *p, const R *sv, const R *t, double rho, const double *scal,
              cudaStream_t s);
// g_d = m(k) i k_d s_d P(p), m = -1/(eps_ref |k|^2), m(0) = 0
template <typename R>
void kgrad_pre(const Grid &g, const R *p, R *g0, R *g1, R *g2, double eps_ref, cudaStream_t s);
// v = sum_d i k_d conj(s_d) w_d (w_d: forward transforms of real fields)
template <typename R>
void kdiv_post(const Grid &g, const R *w0, const R *w1, const R *w2, R *v, cudaStream_t s);
// y = m(k) P(x) (the preconditioner applied to the iterate)
template <typename R>
void kprecond(const Grid &g, const R *x, R *y, double eps_ref, cudaStream_t s);
// the same with 1/eps_ref read from device memory
template <typename R>
void kprecond(const Grid &g, const R *x, R *y, const double *ieps_dev, cudaStream_t s);

// ---- vectors of the flexible GMRES (k-space, read modes) ------------------
constexpr int KVEC_MAX = 34;
struct KVecs {
  const float *p[KVEC_MAX];
};
// partials[b * nv + i] = block b's part of (V_i, w), DOT_BLOCKS blocks
void kmdot(const Grid &g, const KVecs &V, int nv, const float *w, double *partials, cudaStream_t s);
// out[i] = sum over blocks of partials[b * nv + i] (block order)
void kmdot_final(const double *partials, int nv, double *out, cudaStream_t s);
// w += sign * sum_i coef[i] V_i (coef on the device)
void kmaxpy(const Grid &g, float *w, const KVecs &V, int nv, const double *coef, double sign, cudaStream_t s);
// out = w / sqrt(*nrm2)
void kscale_by_norm(const Grid &g, const float *w, float *out, const double *nrm2, cudaStream_t s);
// xt = v + z
void kadd(const Grid &g, const float *v, const float *z, float *xt, cudaStream_t s);
// r = b - w
void ksub(const Grid &g, const float *b, const float *w, float *r, cudaStream_t s);

}  // namespace icep
