// krylov.cuh -- vector kernels of the Poisson solvers: deterministic FP64
// dot products over the real points of padded fields and the fused
// BiCGSTAB updates (van der Vorst 1992; Eigen's loop, used by
// Charge_field2potential_dielectric_LO, operate_dielectric.cxx:542-572).
#pragma once
#include "common.cuh"

namespace icep {

// Device scalar slots written by dot products.
enum ScalarSlot { S_R0V = 0, S_TT, S_TS, S_R0R, S_RR, S_BB, S_AUX0, S_AUX1, S_COUNT };

constexpr int DOT_BLOCKS = 608;  // 4 x 152 SMs
constexpr int DOT_TPB = 256;

// scal[slot + c] = sum over real points of a_c * b_c, c < n (n <= 2); partials
// needs DOT_BLOCKS * 2 doubles.
template <typename R>
void dots(const Grid &g, const R *a0, const R *b0, const R *a1, const R *b1, int n, double *partials, double *scal,
          int slot, cudaStream_t s);

// p = r + beta (p - w v)
template <typename R>
void bicg_p(const Grid &g, R *p, const R *r, const R *v, double beta, double w, cudaStream_t s);
// s = r - alpha v, alpha = rho / scal[S_R0V]
template <typename R>
void bicg_s(const Grid &g, R *sv, const R *r, const R *v, double rho, const double *scal, cudaStream_t s);
// w = ts/tt (0 if tt = 0); x += alpha y + w z; r = s - w t (y, z: the
// preconditioned directions, p and s for the identity preconditioner)
template <typename R>
void bicg_xr(const Grid &g, R *x, R *r, const R *y, const R *z, const R *sv, const R *t, double rho,
             const double *scal, cudaStream_t s);
// y = x (real points), padding zero
template <typename R>
void copy_real(const Grid &g, const R *x, R *y, cudaStream_t s);
// r = b - t (real points)
template <typename R>
void sub_real(const Grid &g, const R *b, const R *t, R *r, cudaStream_t s);
// remove the mean of a real field (mean = scal[slot] / N)
template <typename R>
void sub_mean(const Grid &g, R *a, const double *scal, int slot, cudaStream_t s);
// sum over real points of a (into scal[slot])
template <typename R>
void sum_real(const Grid &g, const R *a, double *partials, double *scal, int slot, cudaStream_t s);
// scal[slot] = sum |a| over the real points
template <typename R>
void sum_abs_real(const Grid &g, const R *a, double *partials, double *scal, int slot, cudaStream_t s);
// type conversion over all NX*NY*NZ_ values
void convert_f2d(long n, const float *x, double *y, cudaStream_t s);
void convert_d2f(long n, const double *x, float *y, cudaStream_t s);
// the same (and a plain copy) where x or y is host memory mapped into the
// device's address space: wide accesses, a strided grid of ~8 blocks per SM
void link_d2f(long n, const double *x, float *y, cudaStream_t s);
void link_f2d(long n, const float *x, double *y, cudaStream_t s);
void link_copy(long n, const double *x, double *y, cudaStream_t s);
// element-wise over all n values (real or k-space arrays): y = (float)(a x);
// y += a (double)x; y = a x + b y
void scale_d2f_all(long n, const double *x, float *y, double a, cudaStream_t s);
void add_f2d_all(long n, const float *x, double *y, double a, cudaStream_t s);
void axpby_all(long n, const double *x, double *y, double a, double b, cudaStream_t s);
// y (double) += a * x (float) on real points
void add_f2d(const Grid &g, const float *x, double *y, double a, cudaStream_t s);
// y (float) = a * x (double) on real points, padding zero
void scale_d2f(const Grid &g, const double *x, float *y, double a, cudaStream_t s);

}  // namespace icep
