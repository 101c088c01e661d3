// fft.cuh -- 3D real FFTs on the reference's padded layout.
//
// Forward (A2a_k, fft_wrapper.h:681-693): kernel exp(-i k.r), unnormalised.
// Inverse (A_k2a, fft_wrapper.h:704-718): 1/N-normalised, with the
// reference's treatment of the kz = 0 and kz = NZ/2 planes (Ooura's
// rdft3dsort reads half of each plane and implies the rest by Hermitian
// symmetry), reproduced by a Hermitian completion of those planes.
//
// Decomposition: z rows (real <-> half complex through an NZ/2-point complex
// FFT), then complex pencils along y and x, each pencil staged in shared
// memory and transformed by a Stockham radix-2 sweep.
#pragma once
#include "common.cuh"

namespace icep {

template <typename R>
struct FFTPlan {
  Grid g;
  cplx<R> *tw_x = nullptr;    // exp(-2 pi i m / NX), m < NX
  cplx<R> *tw_y = nullptr;    // exp(-2 pi i m / NY)
  cplx<R> *tw_z = nullptr;    // exp(-2 pi i m / (NZ/2))
  cplx<R> *tw_post = nullptr; // exp(-2 pi i k / NZ), k <= NZ/2
  // device error word of the kernels with bounded waits (the FP32
  // register-resident plane passes run only when it is set; the owner
  // checks it)
  int *err = nullptr;
};

template <typename R>
int fft_plan_init(FFTPlan<R> &p, const Grid &g, cudaStream_t s);
template <typename R>
void fft_plan_free(FFTPlan<R> &p);

// In-place batched transforms of fb.n fields (device pointers).
template <typename R>
void fft_r2c(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s);
template <typename R>
void fft_c2r(const FFTPlan<R> &p, const FieldBatch<R> &fb, cudaStream_t s);

// The float-float residual's operator core in one sequence: the inverse
// transform of the three fields of fb, each field d times the face
// permittivity 0.5 (eps + eps at the next point along d) (eps: the FP32
// permittivity, real layout), and the forward transform; the z-row passes
// and the product run as one kernel. The same results as fft_c2r, the
// product and fft_r2c (instantiated for the float-float type).
template <typename R>
void fft_c2r_eps_r2c(const FFTPlan<R> &p, const FieldBatch<R> &fb, const float *eps, cudaStream_t s);

// Single passes of the 3D transforms: 0 = z rows + y pencils forward (one
// plane kernel when an x-plane fits in shared memory), 1 = x pencils forward,
// 2 = x pencils inverse, 3 = y pencils + z rows inverse.
template <typename R>
void fft_pass(const FFTPlan<R> &p, const FieldBatch<R> &fb, int pass, cudaStream_t s);

template <typename R>
inline FieldBatch<R> batch(R *a, R *b = nullptr, R *c = nullptr, R *d = nullptr, R *e = nullptr) {
  FieldBatch<R> fb;
  fb.p[0] = a; fb.p[1] = b; fb.p[2] = c; fb.p[3] = d; fb.p[4] = e;
  fb.n = e ? 5 : d ? 4 : c ? 3 : b ? 2 : 1;
  return fb;
}

}  // namespace icep
