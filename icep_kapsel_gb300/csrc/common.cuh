// common.cuh -- shared definitions of the GB300 ICEP library (sm_103a).
//
// Grid fields use the reference's layout [NX][NY][NZ_], NZ_ = 2*(NZ/2+1),
// z fastest; k-space values are interleaved (re,im) pairs in the same buffer
// with kz = 0..NZ/2 (fft_wrapper.h:681-723 in the reference). R is the
// storage/arithmetic type of the fields: double (FP64 mode) or float (the
// FFT/field type of MIXED mode). Particles are always FP64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/icep_gb300.h"

#define ICEP_CUDA_CHECK(call)                                                        \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      fprintf(stderr, "icep_gb300: CUDA error %s at %s:%d\n", cudaGetErrorString(e_), \
              __FILE__, __LINE__);                                                   \
      return ICEP_ERR_CUDA;                                                          \
    }                                                                                \
  } while (0)


namespace icep {

template <typename R>
struct cplx {
  R x, y;
};

// Geometry of one grid (shared by every kernel).
struct Grid {
  int nx, ny, nz;  // mesh
  int hnz;         // NZ/2 + 1 complex values per z row
  int nzp;         // NZ_ = 2*hnz doubles per z row
  int trn[3];      // 2/3-rule limits (N+2)/3
  double wave[3];  // 2 pi / L
  float wavef[3];  // (float)wave: FP32 kernels take it without a per-thread FP64 conversion
  double dx;
  // staggered-grid shifts exp(i dx k_d / 2) as (cos, sin), indexed by the
  // wavenumber index along axis d (i, j or kz); FP64 and FP32 copies
  const double2 *shd[3];
  const float2 *shf[3];
  __host__ __device__ long nf() const { return (long)nx * ny * nzp; }
  __host__ __device__ long nreal() const { return (long)nx * ny * nz; }
  __host__ __device__ long nmodes() const { return (long)nx * ny * hnz; }
};

__host__ __device__ inline long gidx(const Grid &g, int i, int j, int k) {
  return ((long)i * g.ny + j) * g.nzp + k;
}
// real point t (row-major over nx x ny x nz) -> (i, j, k) by shifts and masks:
// every mesh edge is a power of two (checked when a context is created)
__device__ __forceinline__ void real_ijk(const Grid &g, unsigned t, int &i, int &j, int &k) {
  const int lnz = __ffs(g.nz) - 1, lny = __ffs(g.ny) - 1;
  k = (int)(t & (unsigned)(g.nz - 1));
  j = (int)((t >> lnz) & (unsigned)(g.ny - 1));
  i = (int)(t >> (lnz + lny));
}
// mode t of the half spectrum (row-major over nx x ny x hnz) -> (i, j, kz):
// one division by hnz = nz/2 + 1 gives the row i ny + j, split by shift and
// mask (ny a power of two)
__device__ __forceinline__ void mode_ijk3(const Grid &g, unsigned t, int &i, int &j, int &kz) {
  const unsigned row = t / (unsigned)g.hnz;
  kz = (int)(t - row * (unsigned)g.hnz);
  j = (int)(row & (unsigned)(g.ny - 1));
  i = (int)(row >> (__ffs(g.ny) - 1));
}
__host__ __device__ inline int kx_of(const Grid &g, int i) { return (i > g.nx / 2) ? i - g.nx : i; }
__host__ __device__ inline int ky_of(const Grid &g, int j) { return (j > g.ny / 2) ? j - g.ny : j; }
__host__ __device__ inline bool in_two_third(const Grid &g, int i, int j, int kz) {
  int ax = (i <= g.nx / 2) ? i : g.nx - i;
  int ay = (j <= g.ny / 2) ? j : g.ny - j;
  return ax < g.trn[0] && ay < g.trn[1] && kz < g.trn[2];
}

template <typename R>
__host__ __device__ __forceinline__ R wave_of(const Grid &g, int d);
template <>
__host__ __device__ __forceinline__ double wave_of<double>(const Grid &g, int d) { return g.wave[d]; }
template <>
__host__ __device__ __forceinline__ float wave_of<float>(const Grid &g, int d) { return g.wavef[d]; }

__device__ __forceinline__ void shift_of(const Grid &g, int d, int idx, double &c, double &s) {
  const double2 v = g.shd[d][idx];
  c = v.x;
  s = v.y;
}
__device__ __forceinline__ void shift_of(const Grid &g, int d, int idx, float &c, float &s) {
  const float2 v = g.shf[d][idx];
  c = v.x;
  s = v.y;
}

// Weight of k-space mode (i, j, kz) in a real-space inner product taken by
// Parseval over the half spectrum: 0 for the kz = 0 / NZ/2 entries the
// reference's inverse FFT does not read (their values follow by Hermitian
// symmetry), 1 at self-conjugate points (only the real part is read), 2 for
// every other mode.
__host__ __device__ inline int read_weight(const Grid &g, int i, int j, int kz) {
  const int h = g.nz / 2;
  if (kz != 0 && kz != h) return 2;
  const int mi = (g.nx - i) & (g.nx - 1), mj = (g.ny - j) & (g.ny - 1);  // sizes are powers of two
  if (mi == i && mj == j) return 1;
  bool kept;
  if (j >= 1 && j <= g.ny / 2 - 1) kept = true;
  else if (j == 0 || j == g.ny / 2) kept = (i <= g.nx / 2);
  else kept = false;
  if (kz == h) kept = !kept;
  return kept ? 2 : 0;
}

inline unsigned div_up(long a, long b) { return (unsigned)((a + b - 1) / b); }

// Number of kernels this library has launched (all contexts); read by
// icep_kernel_launches() so that a benchmark can report its launch count.
extern unsigned long long g_kernel_launches;
inline void count_launch() { __atomic_fetch_add(&g_kernel_launches, 1ULL, __ATOMIC_RELAXED); }
// Algorithmic bytes of the kernels launched (all contexts; read by
// icep_algorithmic_bytes()): each launch adds its external inputs and
// outputs -- one grid field of NX NY NZ values of its type per field read or
// written (a half spectrum counts as one field, an in-place update as one
// read and one write), one field per field and pass of a 3D transform (the
// 2 N s of a transform over its two passes), Np n_dom s per component of a
// scatter (read and write: 2) or gather -- so that a step's total over its
// time is its roofline figure.
extern unsigned long long g_alg_bytes;
inline void count_launch(double bytes) {
  count_launch();
  if (bytes > 0) __atomic_fetch_add(&g_alg_bytes, (unsigned long long)(bytes + 0.5), __ATOMIC_RELAXED);
}
// bytes of `nfields` grid fields of element type R
template <typename R>
inline double fld(const Grid &g, double nfields) { return nfields * (double)g.nreal() * sizeof(R); }
// number of distinct non-null operands (a dot product reads each field once)
inline double ndistinct(const void *a, const void *b, const void *c = nullptr, const void *d = nullptr) {
  const void *v[4] = {a, b, c, d};
  int n = 0;
  for (int i = 0; i < 4; i++) {
    if (!v[i]) continue;
    bool seen = false;
    for (int j = 0; j < i; j++) seen = seen || (v[j] == v[i]);
    if (!seen) n++;
  }
  return (double)n;
}

// Field slots of a context (ids shared with the oracle and the C-ABI).
enum FieldId {
  F_ZETA0 = 0, F_ZETA1, F_U0, F_U1, F_U2, F_UP0, F_UP1, F_UP2, F_PHI, F_PHI_SUM,
  F_F0, F_F1, F_F2, F_POT, F_EPS, F_GE0, F_GE1, F_GE2, F_C0, F_C1, F_RHO, F_WORK,
  F_SN0, F_SN1, F_SN2, F_NS0_0, F_NS0_1, F_NS1_0, F_NS1_1, F_CRHS0, F_CRHS1,
  F_WV1, F_WV3_0, F_WV3_1, F_WV3_2,
  // Krylov work vectors (padded fields)
  F_KR, F_KR0, F_KP, F_KV, F_KS, F_KT, F_KX, F_KB, F_KY, F_KZ,
  // face permittivities of the fused k-space operator
  F_EF0, F_EF1, F_EF2,
  // the fused operator's fourth work field (its z component)
  F_WV3_3,
  F_COUNT
};

// Up to 5 fields transformed by one batched launch.
template <typename R>
struct FieldBatch {
  R *p[5];
  int n;
};

}  // namespace icep
