// refine.cuh -- the FP64-accurate half of the MIXED Poisson solve in
// float-float arithmetic (dfloat.cuh) on the FP32 pipes.
//
// The MIXED solve refines the potential's half spectrum x^ against the true
// residual r^ = b^ - A x^ of the reference operator
//   A x = D^-.(eps_face D^+ x)      (Ax, operate_dielectric.cxx:485-522)
//   b   = D^-.(eps_face E_ext) - rho (Build_rhs, operate_dielectric.cxx:524-540)
// with eps_face_d = (eps + eps shifted by one point along d)/2 and the
// staggered spectral derivatives D^+_d = i k_d exp(+i dx k_d/2),
// D^-_d = i k_d exp(-i dx k_d/2). x^, b^, r^ and the three face fields are
// float-float vectors (hi, lo pairs in the reference's padded layout, one
// 8-byte number per double of the FP64 layout); the transforms are the
// float-float FFT (fft_df.cu). Norms are Parseval sums over the read modes
// (weights of read_weight), scaled by 1/N like the inner solver's dots.
#pragma once
#include "dfloat.cuh"
#include "fft.cuh"

namespace icep {

// Per-axis multipliers of the staggered gradient, D^+_d(q) = (re, im) as
// float-float (re.hi, re.lo, im.hi, im.lo), q the wavenumber index along d
// (i, j or kz); the divergence multiplier is D^-_d = -conj(D^+_d).
struct RefineTables {
  float4 *gd[3] = {nullptr, nullptr, nullptr};
  void *mem = nullptr;
  int init(const Grid &g, cudaStream_t s);
  void free_all();
};

// out = (dfl)a (exact), n numbers
void rf_from_f32(long n, const float *a, dfl *out, cudaStream_t s);
// out = (float)(a * scale)
void rf_to_f32(long n, const dfl *a, float *out, double scale, cudaStream_t s);
// the same with the FP32 factor read from device memory
void rf_to_f32(long n, const dfl *a, float *out, const float *scale_dev, cudaStream_t s);
// out = (double)a
void rf_to_f64(long n, const dfl *a, double *out, cudaStream_t s);
// *flag = 1 if the n doubles a and b differ in any bit, else 0 (device int)
void rf_differs(long n, const double *a, const double *b, int *flag, cudaStream_t s);
// x += a * d (a a host double, d FP32)
void rf_add_f32(long n, const float *d, dfl *x, double a, cudaStream_t s);
// the same with a read from device memory as a float-float pair (hi, lo)
void rf_add_f32(long n, const float *d, dfl *x, const float2 *a_dev, cudaStream_t s);
// x <- 2 x - xp and xp <- x in place (linear extrapolation in time)
void rf_extrapolate_shift(long n, dfl *x, dfl *xp, cudaStream_t s);
// x = 0 if *flag (a device double) is non-zero
void rf_zero_if(long n, dfl *x, const double *flag, cudaStream_t s);
// w_d = D^+_d x^ (k-space, d = 0..2)
void rf_grad(const Grid &g, const RefineTables &t, const dfl *x, dfl *w0, dfl *w1, dfl *w2, cudaStream_t s);
// w_d *= eps_face_d (real points; eps is the FP32 permittivity)
void rf_eps_face_mul(const Grid &g, dfl *w0, dfl *w1, dfl *w2, const float *eps, cudaStream_t s);
// w_d = eps_face_d * e_d for the components with use[d] (real points)
void rf_eps_face_e(const Grid &g, dfl *w0, dfl *w1, dfl *w2, const float *eps, const double *e, const bool *use,
                   cudaStream_t s);
// k-space combination of the divergence sum_d D^-_d w_d (components with
// use[d]) and a base vector:
//   RF_RESIDUAL: out = base - div          (r^ = b^ - A x^)
//   RF_RHS:      out = div - base, k = 0 mode zeroed  (b^ = D^-.(eps_face E) - rho^)
// and the Parseval norm |out|^2 / N over the read modes into scal[slot]
// (partials: DOT_BLOCKS * 2 doubles). Squares are summed in FP32 after a
// power-of-two prescale `prescale` (chosen from |b| by the caller so that
// no square under- or overflows), per thread, then in FP64 across threads;
// acc64 sums them in FP64 instead (no prescale needed).
enum { RF_RESIDUAL = 0, RF_RHS = 1 };
// prescale_dev (if given, FP32 sums only) replaces prescale by a value
// formed on the device.
void rf_div_combine(const Grid &g, const RefineTables &t, const dfl *w0, const dfl *w1, const dfl *w2,
                    const bool *use, const dfl *base, dfl *out, int mode, float prescale, bool acc64,
                    double *partials, double *scal, int slot, cudaStream_t s, const float *prescale_dev = nullptr);

}  // namespace icep
